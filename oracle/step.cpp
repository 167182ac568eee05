// One simulation time step of the rigid IPC problem (test infrastructure).
//
// Restates DistanceBarrierRBProblem::simulation_step
// (src/problems/distance_barrier_rb_problem.cpp:118-143) for the default
// settings (implicit Euler, IPC solver with velocity convergence, one friction
// lagging iteration, no kinematic bodies):
//  * update_constraints (:145-166): constraint set at the start-of-step poses
//    x0 and, with friction, the lagged friction constraints (normal forces
//    with the current barrier stiffness);
//  * IPCSolver::init_solve (src/solvers/ipc_solver.cpp:36-65): the initial
//    barrier stiffness from the energy and barrier gradients at x0 and the
//    initial minimum distance;
//  * NewtonSolver::solve (src/solvers/newton_solver.cpp:158-300): objective
//    E/m + kappa/m B + D/m (compute_objective, :633-703) over the free
//    degrees of freedom, regularised Newton direction
//    (compute_regularized_direction, :421-478; a dense LDL^T stands in for the
//    sparse one), the velocity convergence test (:95-140), a line search over
//    [0, min(toi, 1)] halving the step until the objective decreases
//    (:302-418), the gradient fallback, and the adaptive stiffness update
//    after each step (ipc_solver.cpp:67-89);
//  * take_step (:488-626): implicit-Euler velocity and Qdot updates.
// The two ipc-toolkit functions used by the solver are restated from the
// published adaptive-stiffness scheme of Li et al. 2020 (IPC, sec. 4.3):
// kappa0 = argmin |grad E + kappa grad B| clamped to [kappa_min, 100 kappa_min]
// with kappa_min = scale * m / (4 d0 b''(d0)), d0 = (1e-8 bbox)^2; kappa
// doubles while the minimum distance keeps shrinking below 1e-9 bbox.
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

#include "oracle.hpp"

namespace orc {

namespace {

double barrier_hessian_d(double d, double s)
{
    if (d <= 0.0 || d >= s) return 0.0;
    double sd = s / d;
    return (sd + 2) * sd - 2 * std::log(d / s) - 3;
}

} // namespace

// squared distance of one constraint (the distance its barrier uses)
double constraint_sqdist(const Constraint& c, const std::vector<double>& V)
{
    auto P = [&](int i) { return &V[3 * c.v[i]]; };
    switch (c.type) {
    case C_VV: return point_point_sqdist(P(0), P(1));
    case C_EV: return point_line_sqdist(P(0), P(1), P(2));
    case C_EE: return edge_edge_sqdist(P(0), P(1), P(2), P(3));
    default: return point_plane_sqdist(P(0), P(1), P(2), P(3));
    }
}

namespace {

// dense LDL^T (no pivoting) of a symmetric matrix; false on a zero pivot
bool ldlt_solve(int n, std::vector<double> A, const std::vector<double>& b,
                std::vector<double>& x)
{
    std::vector<double> D(n);
    for (int j = 0; j < n; j++) {
        double d = A[j * n + j];
        for (int k = 0; k < j; k++) d -= A[j * n + k] * A[j * n + k] * D[k];
        if (!(std::fabs(d) > 0) || !std::isfinite(d)) return false;
        D[j] = d;
        for (int i = j + 1; i < n; i++) {
            double s = A[i * n + j];
            for (int k = 0; k < j; k++) s -= A[i * n + k] * A[j * n + k] * D[k];
            A[i * n + j] = s / d;
        }
    }
    x = b;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < i; k++) x[i] -= A[i * n + k] * x[k];
    for (int i = 0; i < n; i++) x[i] /= D[i];
    for (int i = n - 1; i >= 0; i--)
        for (int k = i + 1; k < n; k++) x[i] -= A[k * n + i] * x[k];
    for (double v : x)
        if (!std::isfinite(v)) return false;
    return true;
}

struct Problem {
    const Scene& s;
    const std::vector<BodyState>& bodies;
    const SimParams& p;
    double kappa, kappa_max = 0;
    std::vector<FrictionConstraint> fric;
    std::vector<double> x0;
    SimStats* st;
    double s_average_mass;
    // augmented Lagrangian of the kinematic bodies (init_augmented_lagrangian,
    // distance_barrier_rb_problem.cpp:190-235): targets x_pred = x0 + h v,
    // penalties, multipliers (3 per body linear, 3 x 3 angular), and whether
    // the linear / angular constraints are satisfied
    std::vector<double> x_pred, lam, Lam;
    double kq = 1e3, kQ = 1e3;
    bool sat_q = false, sat_Q = false, has_kinematic = false;

    Problem(const Scene& s_, const std::vector<BodyState>& b, const SimParams& p_, double k,
            SimStats* st_)
        : s(s_), bodies(b), p(p_), kappa(k), st(st_), s_average_mass(p_.average_mass)
    {
    }

    int n() const { return 6 * s.nb; }

    std::vector<Constraint> constraints(const double* x) const
    {
        Candidates cand;
        detect_candidates(s, x, x, false, (p.dhat + p.dmin) / 2, false, cand);
        std::vector<double> V;
        world_vertices(s, x, V);
        std::vector<Constraint> cs;
        construct_constraint_set(s, cand, V, p.dhat, p.dmin, cs);
        return cs;
    }

    double min_distance(const double* x) const
    {
        std::vector<Constraint> cs = constraints(x);
        if (cs.empty()) return -1;
        std::vector<double> V;
        world_vertices(s, x, V);
        double m = INFINITY;
        for (const auto& c : cs) m = std::min(m, constraint_sqdist(c, V));
        return std::isfinite(m) ? std::sqrt(m) : -1;
    }

    // body energy term (not divided by the average mass)
    double energy_term(const double* x, std::vector<double>* g, std::vector<double>* H) const
    {
        const int N = n();
        if (g) g->assign(N, 0.0);
        if (H) H->assign((size_t)N * N, 0.0);
        double e = 0;
        for (int b = 0; b < s.nb; b++) {
            if (bodies[b].type != 2) continue;
            double gb[6], hb[36];
            e += body_energy(bodies[b], x + 6 * b, p.gravity, p.h, gb, hb);
            // PSD projection of the position block (:765-768)
            double P3[9], Q3[9];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) P3[3 * r + c] = hb[6 * r + c];
            project_to_psd(3, P3, Q3);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) hb[6 * r + c] = Q3[3 * r + c];
            if (g)
                for (int k = 0; k < 6; k++) (*g)[6 * b + k] += gb[k];
            if (H)
                for (int r = 0; r < 6; r++)
                    for (int c = 0; c < 6; c++)
                        (*H)[(size_t)(6 * b + r) * N + 6 * b + c] += hb[6 * r + c];
        }
        return e;
    }

    static void add_bsr(const BSR& h, int N, double scale, std::vector<double>& H)
    {
        const int nb = (int)h.row_ptr.size() - 1;
        for (int r = 0; r < nb; r++)
            for (int k = h.row_ptr[r]; k < h.row_ptr[r + 1]; k++)
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++)
                        H[(size_t)(6 * r + i) * N + 6 * h.col[k] + j] += scale * h.val[36 * k + 6 * i + j];
    }

    static void jhalf(const double* I, double J[3], double Js[3])
    {
        J[0] = 0.5 * (-I[0] + I[1] + I[2]);
        J[1] = 0.5 * (I[0] - I[1] + I[2]);
        J[2] = 0.5 * (I[0] + I[1] - I[2]);
        for (int k = 0; k < 3; k++) Js[k] = std::sqrt(std::max(J[k], 0.0));
    }

    // compute_augmented_lagrangian (:946-1109), added to g and H (unscaled);
    // zero once every kinematic constraint is satisfied
    double augmented_lagrangian(const double* x, std::vector<double>* g, std::vector<double>* H) const
    {
        if (!has_kinematic || (sat_q && sat_Q)) return 0.0;
        const int N = n();
        double e = 0;
        for (int b = 0; b < s.nb; b++) {
            if (bodies[b].type != 1) continue;
            const double m = bodies[b].mass, sm = std::sqrt(m);
            const double* q = x + 6 * b;
            const double* qp = &x_pred[6 * b];
            for (int i = 0; i < 3; i++) {
                const double d = q[i] - qp[i];
                e += kq / 2 * m * d * d - sm * lam[3 * b + i] * d;
                if (g) (*g)[6 * b + i] += kq * m * d - sm * lam[3 * b + i];
                if (H) (*H)[(size_t)(6 * b + i) * N + 6 * b + i] += kq * m;
            }
            double J[3], Js[3];
            jhalf(bodies[b].moment, J, Js);
            double Qp[9], Qv[9], dQ[27];
            rotation_matrix(qp + 3, Qp);
            rotation_matrix(q + 3, Qv);
            rotation_matrix_jacobian(q + 3, dQ);
            // kQ/2 tr((Q - Qp) J (Q - Qp)^T) - tr(Lam^T (Q - Qp) Js)
            double ga[3] = { 0, 0, 0 };
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) {
                    const double d = Qv[3 * i + k] - Qp[3 * i + k];
                    const double L = Lam[9 * b + 3 * i + k];
                    e += kQ / 2 * J[k] * d * d - L * d * Js[k];
                    const double c = kQ * J[k] * d - L * Js[k];
                    for (int a = 0; a < 3; a++) ga[a] += c * dQ[9 * a + 3 * i + k];
                }
            if (g)
                for (int a = 0; a < 3; a++) (*g)[6 * b + 3 + a] += ga[a];
            if (H) {
                double d2Q[81];
                rotation_matrix_hessian(q + 3, d2Q);
                for (int a = 0; a < 3; a++)
                    for (int c2 = 0; c2 < 3; c2++) {
                        double h = 0;
                        for (int i = 0; i < 3; i++)
                            for (int k = 0; k < 3; k++) {
                                const double d = Qv[3 * i + k] - Qp[3 * i + k];
                                const double c = kQ * J[k] * d - Lam[9 * b + 3 * i + k] * Js[k];
                                h += kQ * J[k] * dQ[9 * a + 3 * i + k] * dQ[9 * c2 + 3 * i + k]
                                    + c * d2Q[27 * a + 9 * c2 + 3 * i + k];
                            }
                        (*H)[(size_t)(6 * b + 3 + a) * N + 6 * b + 3 + c2] += h;
                    }
            }
        }
        return e;
    }

    // compute_{linear,angular}_augment_lagrangian_progress (:265-337)
    void al_progress(const double* x, double& eq, double& eQ) const
    {
        double aq = 0, bq = 0, aQ = 0, bQ = 0;
        for (int b = 0; b < s.nb; b++) {
            if (bodies[b].type != 1) continue;
            for (int i = 0; i < 3; i++) {
                aq += (x_pred[6 * b + i] - x[6 * b + i]) * (x_pred[6 * b + i] - x[6 * b + i]);
                bq += (x_pred[6 * b + i] - x0[6 * b + i]) * (x_pred[6 * b + i] - x0[6 * b + i]);
            }
            double Qp[9], Qv[9], Q0[9];
            rotation_matrix(&x_pred[6 * b + 3], Qp);
            rotation_matrix(x + 6 * b + 3, Qv);
            rotation_matrix(&x0[6 * b + 3], Q0);
            for (int k = 0; k < 9; k++) {
                aQ += (Qv[k] - Qp[k]) * (Qv[k] - Qp[k]);
                bQ += (Q0[k] - Qp[k]) * (Q0[k] - Qp[k]);
            }
        }
        eq = (aq == 0 && bq == 0) ? 1.0 : 1 - std::sqrt(aq / (bq == 0 ? 1 : bq));
        eQ = (aQ == 0 && bQ == 0) ? 1.0 : 1 - std::sqrt(aQ / (bQ == 0 ? 1 : bQ));
    }

    bool al_satisfied(const double* x) const
    {
        if (!has_kinematic) return true;
        double eq, eQ;
        al_progress(x, eq, eQ);
        return eq >= 0.999 && eQ >= 0.999;
    }

    // update_augmented_lagrangian (:339-423)
    void al_update(const double* x)
    {
        double eq, eQ;
        al_progress(x, eq, eQ);
        if (eq >= 0.999) {
            sat_q = true;
        } else if (eq < 0.99 && kq < 1e8) {
            kq *= 2;
        } else {
            for (int b = 0; b < s.nb; b++)
                if (bodies[b].type == 1)
                    for (int i = 0; i < 3; i++)
                        lam[3 * b + i] -= kq * std::sqrt(bodies[b].mass) * (x[6 * b + i] - x_pred[6 * b + i]);
        }
        if (eQ >= 0.999) {
            sat_Q = true;
        } else if (eQ < 0.99 && kQ < 1e8) {
            kQ *= 2;
        } else {
            for (int b = 0; b < s.nb; b++) {
                if (bodies[b].type != 1) continue;
                double Qp[9], Qv[9], J[3], Js[3];
                rotation_matrix(&x_pred[6 * b + 3], Qp);
                rotation_matrix(x + 6 * b + 3, Qv);
                jhalf(bodies[b].moment, J, Js);
                for (int i = 0; i < 3; i++)
                    for (int k = 0; k < 3; k++)
                        Lam[9 * b + 3 * i + k] -= kQ * (Qv[3 * i + k] - Qp[3 * i + k]) * Js[k];
            }
        }
    }

    // compute_objective (:633-703)
    double objective(const double* x, std::vector<double>* g, std::vector<double>* H) const
    {
        const int N = n();
        const double m = s_average_mass;
        double f = energy_term(x, g, H);
        f += augmented_lagrangian(x, g, H);
        f /= m;
        if (g)
            for (double& v : *g) v /= m;
        if (H)
            for (double& v : *H) v /= m;
        std::vector<Constraint> cs = constraints(x);
        if (g || H) {
            std::vector<double> gb;
            BSR hb;
            double B = barrier_term(s, x, cs, p.dhat, p.dmin, gb, hb, true);
            f += kappa / m * B;
            if (g)
                for (int k = 0; k < N; k++) (*g)[k] += kappa / m * gb[k];
            if (H) add_bsr(hb, N, kappa / m, *H);
        } else {
            f += kappa / m * barrier_energy(s, x, cs, p.dhat, p.dmin);
        }
        if (p.mu > 0 && !fric.empty()) {
            std::vector<double> gd;
            BSR hd;
            double D = friction_term(s, x, x0.data(), fric, p.mu, p.epsv * p.h, gd, hd, true);
            f += D / m;
            if (g)
                for (int k = 0; k < N; k++) (*g)[k] += gd[k] / m;
            if (H) add_bsr(hd, N, 1.0 / m, *H);
        }
        if (st) st->objective_evals++;
        return f;
    }

    double toi(const double* x, const double* x1) const
    {
        Candidates cand;
        detect_candidates(s, x, x1, true, p.dmin / 2, false, cand);
        const int nt = std::max(1, (int)std::thread::hardware_concurrency());
        if (p.trajectory == 1) return pl_earliest_toi(s, x, x1, cand, p.dmin, nt, nullptr, nullptr);
        return earliest_toi(s, x, x1, cand, 1e-4, nt, nullptr, nullptr);
    }
};

} // namespace

void simulation_step(const Scene& s, std::vector<BodyState>& bodies, const SimParams& p,
                     double& kappa, SimStats* st, StepRecord* rec)
{
    const int nb = s.nb, N = 6 * nb;
    Problem pr(s, bodies, p, kappa, st);
    pr.x0.resize(N);
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 6; k++) pr.x0[6 * b + k] = bodies[b].pose_t0[k];
    const double* x0 = pr.x0.data();
    // init_augmented_lagrangian (distance_barrier_rb_problem.cpp:190-234):
    // kinematic targets, the front of the body's pose list or x0 + h v
    pr.x_pred = pr.x0;
    pr.lam.assign(3 * (size_t)nb, 0.0);
    pr.Lam.assign(9 * (size_t)nb, 0.0);
    for (int b = 0; b < nb; b++)
        if (bodies[b].type == 1) {
            pr.has_kinematic = true;
            for (int k = 0; k < 6; k++)
                pr.x_pred[6 * b + k] = bodies[b].has_target ? bodies[b].kin_target[k]
                                                            : pr.x0[6 * b + k] + p.h * bodies[b].vel_t0[k];
        }

    // update_constraints: lagged friction at x0 with the current stiffness
    if (p.mu > 0) {
        std::vector<Constraint> cs = pr.constraints(x0);
        std::vector<double> V0;
        world_vertices(s, x0, V0);
        construct_friction_constraints(s, cs, V0, p.dhat, 0.0, pr.kappa, pr.fric);
    }

    // IPCSolver::init_solve
    double dk = 0;  // d kappa / d kappa0
    {
        std::vector<double> gE, gB;
        pr.energy_term(x0, &gE, nullptr);
        BSR hb;
        std::vector<Constraint> cs = pr.constraints(x0);
        barrier_term(s, x0, cs, p.dhat, p.dmin, gB, hb, false);
        const double dmin = p.dmin;
        double d0 = 1e-8 * p.bbox_diagonal + dmin;
        d0 *= d0;
        const double sb = 2 * dmin * p.dhat + p.dhat * p.dhat;
        if (d0 - dmin * dmin >= sb) d0 = dmin * p.dhat + 0.5 * p.dhat * p.dhat;
        double kmin = 4 * d0 * barrier_hessian_d(d0 - dmin * dmin, sb);
        kmin = p.min_barrier_stiffness_scale * p.average_mass / kmin;
        pr.kappa_max = 100 * kmin;
        double gg = 0, ge = 0;
        for (int k = 0; k < N; k++) {
            gg += gB[k] * gB[k];
            ge += gB[k] * gE[k];
        }
        double k0 = gg > 0 ? -ge / gg : 1.0;
        pr.kappa = std::min(pr.kappa_max, std::max(kmin, k0));
        dk = (gg > 0 && k0 > kmin && k0 < pr.kappa_max) ? 1.0 : 0.0;
    }
    double prev_min_distance = pr.min_distance(x0);

    // free degrees of freedom
    std::vector<int> free_dof;
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 6; k++)
            if (!bodies[b].fixed[k]) free_dof.push_back(6 * b + k);
    const int nf = (int)free_dof.size();

    std::vector<double> x = pr.x0, g, H, dir(N, 0.0), gdir(N, 0.0);
    double coeff = 0;
    bool energy_converged = false;
    int it = 0;
    for (; it < p.max_newton_iterations; it++) {
        double fx = pr.objective(x.data(), &g, &H);
        std::vector<double> gf(nf), Hf((size_t)nf * nf), df;
        for (int i = 0; i < nf; i++) {
            gf[i] = g[free_dof[i]];
            for (int j = 0; j < nf; j++) Hf[(size_t)i * nf + j] = H[(size_t)free_dof[i] * N + free_dof[j]];
        }
        // compute_regularized_direction
        bool ok = false;
        while (!ok) {
            std::vector<double> Hr = Hf, mg(nf);
            if (coeff > 0)
                for (int i = 0; i < nf; i++) Hr[(size_t)i * nf + i] += coeff;
            for (int i = 0; i < nf; i++) mg[i] = -gf[i];
            // a failed factorisation counts as a failed solve: regularise
            ok = ldlt_solve(nf, Hr, mg, df);
            double gd = 0;
            if (!ok) df = mg;
            for (int i = 0; i < nf; i++) gd += gf[i] * df[i];
            ok = ok && gd <= 0;
            if (ok) {
                coeff /= 2;
                if (coeff < 1e-8) coeff = 0;
            } else {
                coeff = std::max(2 * coeff, 1e-8);
                if (!std::isfinite(coeff)) break;
            }
        }
        if (!ok) break;
        std::fill(dir.begin(), dir.end(), 0.0);
        std::fill(gdir.begin(), gdir.end(), 0.0);
        for (int i = 0; i < nf; i++) {
            dir[free_dof[i]] = df[i];
            gdir[free_dof[i]] = gf[i];
        }
        // velocity convergence
        if (it > 0) {
            std::vector<double> V, V1, x1(N);
            for (int k = 0; k < N; k++) x1[k] = x[k] + dir[k];
            world_vertices(s, x.data(), V);
            world_vertices(s, x1.data(), V1);
            double m = 0;
            for (size_t k = 0; k < V.size(); k++) m = std::max(m, std::fabs(V1[k] - V[k]));
            double tol = p.velocity_conv_tol * (p.velocity_conv_tol_abs ? 1.0 : p.bbox_diagonal);
            // converged (:95-156): the velocity test and the kinematic
            // equality constraints
            energy_converged = m / p.h <= tol;
            if (energy_converged && pr.al_satisfied(x.data())) break;
        }
        auto line_search = [&](const std::vector<double>& d, double& alpha) {
            double gd = 0;
            for (int k = 0; k < N; k++) gd += gdir[k] * d[k];
            double lb = std::min(p.line_search_lower_bound / std::sqrt(std::fabs(gd)), 1e-1);
            std::vector<double> x1(N);
            for (int k = 0; k < N; k++) x1[k] = x[k] + d[k];
            double tmax = pr.toi(x.data(), x1.data());
            tmax = std::min(tmax < 1.0 ? p.ccd_rescale * tmax : tmax, 1.0);
            if (st) st->ccd_calls++;
            alpha = std::min(1.0, tmax);
            while (std::isfinite(lb) && alpha >= lb) {
                for (int k = 0; k < N; k++) x1[k] = x[k] + alpha * d[k];
                double fxi = pr.objective(x1.data(), nullptr, nullptr);
                if (fxi < fx) return true;
                alpha /= 2.0;
            }
            return false;
        };
        double alpha = 1;
        bool found = line_search(dir, alpha);
        if (!found) {
            for (int k = 0; k < N; k++) dir[k] = -gdir[k];
            alpha = 1;
            if (!line_search(dir, alpha)) break;
        }
        for (int k = 0; k < N; k++) x[k] += alpha * dir[k];
        if (st) st->newton_steps++;
        // NewtonSolver::post_step_update (:606-612): augmented Lagrangian
        if (energy_converged && !pr.al_satisfied(x.data())) pr.al_update(x.data());
        // IPCSolver::post_step_update: adaptive stiffness
        double md = pr.min_distance(x.data());
        double eps = p.dhat_epsilon * (p.bbox_diagonal + p.dmin);
        if (prev_min_distance < eps && md < eps && md < prev_min_distance) {
            dk = 2 * pr.kappa < pr.kappa_max ? 2 * dk : 0.0;
            pr.kappa = std::min(pr.kappa_max, 2 * pr.kappa);
        }
        prev_min_distance = md;
    }
    if (st) st->newton_iterations += it;

    // optional polish (not in the reference): full Newton steps with the
    // unprojected Hessian while they keep contracting and the CCD admits the
    // full step.  The line search's test f(x + a d) < f(x) stalls where the
    // decrease falls below the rounding of f (|dx| ~ sqrt(eps)); these steps
    // take the solution to the rounding of the gradient instead, which the
    // adjoint and finite differences of the trajectory need.
    double prev_step = INFINITY;
    for (int k = 0; k < p.newton_polish; k++) {
        std::vector<double> gp, Hp;
        {
            const double m = pr.s_average_mass;
            pr.energy_term(x.data(), &gp, &Hp);
            pr.augmented_lagrangian(x.data(), &gp, &Hp);
            for (double& v : gp) v /= m;
            for (double& v : Hp) v /= m;
            std::vector<Constraint> cs = pr.constraints(x.data());
            std::vector<double> gb;
            BSR hb;
            barrier_term(s, x.data(), cs, p.dhat, p.dmin, gb, hb, false);
            for (int i = 0; i < N; i++) gp[i] += pr.kappa / m * gb[i];
            Problem::add_bsr(hb, N, pr.kappa / m, Hp);
        }
        std::vector<double> gf(nf), Hf((size_t)nf * nf), df;
        for (int i = 0; i < nf; i++) {
            gf[i] = -gp[free_dof[i]];
            for (int j = 0; j < nf; j++) Hf[(size_t)i * nf + j] = Hp[(size_t)free_dof[i] * N + free_dof[j]];
        }
        if (!ldlt_solve(nf, Hf, gf, df)) break;
        double step = 0, gd = 0;
        for (int i = 0; i < nf; i++) {
            step = std::max(step, std::fabs(df[i]));
            gd -= gf[i] * df[i];
        }
        if (!(step > 0) || gd > 0 || step >= 0.5 * prev_step) break;
        std::vector<double> x1 = x;
        for (int i = 0; i < nf; i++) x1[free_dof[i]] += df[i];
        if (pr.toi(x.data(), x1.data()) < 1.0) break;
        x = x1;
        prev_step = step;
        if (st) st->newton_steps++;
    }

    if (rec) {
        rec->x = x;
        rec->kappa = pr.kappa;
        rec->dkappa_dk0 = dk;
    }

    // take_step: implicit Euler velocities
    for (int b = 0; b < nb; b++) {
        BodyState& B = bodies[b];
        if (B.type != 2) {
            // set_rb_poses moves every body; only dynamic ones get velocities
            for (int k = 0; k < 6; k++) B.pose_t0[k] = x[6 * b + k];
            continue;
        }
        double Q[9], Qp[9];
        rotation_matrix(&x[6 * b + 3], Q);
        rotation_matrix(&B.pose_t0[3], Qp);
        for (int k = 0; k < 3; k++) B.vel_t0[k] = (x[6 * b + k] - B.pose_t0[k]) / p.h;
        for (int k = 0; k < 9; k++) B.Qdot[k] = (Q[k] - Qp[k]) / p.h;
        for (int k = 0; k < 3; k++)
            if (B.fixed[k]) B.vel_t0[k] = 0;
        for (int k = 0; k < 6; k++) B.pose_t0[k] = x[6 * b + k];
    }
    kappa = pr.kappa;
}

// ---------------------------------------------------------------------------
// Adjoint of one step (new: the reference has no adjoint).  The step maps the
// state s = (x0, v, Qdot) to x* = argmin f(x; s) over the free dofs, with
// f = E(x; s) / m + kappa / m B(x) (no friction), then s' = (x*, (x* - x0) /
// h, (R(theta*) - R(theta0)) / h).  With the gradient of f zero at x*:
//   H_FF lambda = dL/dx*_F,   dL/ds = dL/ds|direct - (1/m) E_xs^T lambda,
// where H is the unprojected Hessian of f at x*; fixed dofs keep x0, so they
// pass dL/dx*_C - (H lambda)_C back to x0.  The initial stiffness kappa0 =
// -gE.gB / gB.gB at x0 (inside its clamp) depends on s as well:
//   dL/dkappa = -(1/m) lambda . gB(x*),
//   dkappa0/ds = -(1/gB.gB) [P^T (H_B (gE + 2 kappa0 gB) + H_E gB) + E_xs^T gB]
// at x0 (P: the pose part of s).
bool adjoint_step(const Scene& s, const std::vector<BodyState>& pre, const SimParams& p,
                  const StepRecord& rec, const AdjointState& in, AdjointState& out)
{
    const int nb = s.nb, N = 6 * nb;
    for (int b = 0; b < nb; b++)
        if (pre[b].type == 1) return false;  // kinematic bodies are not differentiated
    const double M = p.average_mass, h = p.h;
    const double* x = rec.x.data();
    out.pose.assign(N, 0.0);
    out.vel.assign(N, 0.0);
    out.Qdot.assign(9 * (size_t)nb, 0.0);
    std::vector<double> xbar(N, 0.0);
    for (int b = 0; b < nb; b++) {
        const BodyState& B = pre[b];
        for (int k = 0; k < 6; k++) xbar[6 * b + k] = in.pose[6 * b + k];
        if (B.type != 2) {
            for (int k = 0; k < 6; k++) out.vel[6 * b + k] += in.vel[6 * b + k];
            for (int k = 0; k < 9; k++) out.Qdot[9 * b + k] += in.Qdot[9 * b + k];
            continue;
        }
        for (int k = 0; k < 3; k++) {
            if (!B.fixed[k]) {
                xbar[6 * b + k] += in.vel[6 * b + k] / h;
                out.pose[6 * b + k] -= in.vel[6 * b + k] / h;
            }
            out.vel[6 * b + 3 + k] += in.vel[6 * b + 3 + k];  // angular velocity is kept
        }
        double dR1[27], dR0[27];
        rotation_matrix_jacobian(x + 6 * b + 3, dR1);
        rotation_matrix_jacobian(B.pose_t0 + 3, dR0);
        for (int a = 0; a < 3; a++) {
            double s1 = 0, s0 = 0;
            for (int k = 0; k < 9; k++) {
                s1 += in.Qdot[9 * b + k] * dR1[9 * a + k];
                s0 += in.Qdot[9 * b + k] * dR0[9 * a + k];
            }
            xbar[6 * b + 3 + a] += s1 / h;
            out.pose[6 * b + 3 + a] -= s0 / h;
        }
    }

    Problem pr(s, pre, p, rec.kappa, nullptr);
    // unprojected Hessian of f at x*
    std::vector<double> H((size_t)N * N, 0.0), gBx;
    for (int b = 0; b < nb; b++) {
        double g6[6], h36[36];
        body_energy(pre[b], x + 6 * b, p.gravity, h, g6, h36);
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++) H[(size_t)(6 * b + r) * N + 6 * b + c] = h36[6 * r + c] / M;
    }
    {
        BSR hb;
        std::vector<Constraint> cs = pr.constraints(x);
        barrier_term(s, x, cs, p.dhat, p.dmin, gBx, hb, false);
        Problem::add_bsr(hb, N, rec.kappa / M, H);
    }
    std::vector<int> F;
    std::vector<char> is_free(N, 0);
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 6; k++)
            if (!pre[b].fixed[k]) {
                F.push_back(6 * b + k);
                is_free[6 * b + k] = 1;
            }
    const int nf = (int)F.size();
    std::vector<double> HF((size_t)nf * nf), rhs(nf), lf;
    for (int i = 0; i < nf; i++) {
        rhs[i] = xbar[F[i]];
        for (int j = 0; j < nf; j++) HF[(size_t)i * nf + j] = H[(size_t)F[i] * N + F[j]];
    }
    if (nf > 0 && !ldlt_solve(nf, HF, rhs, lf)) return false;
    std::vector<double> lam(N, 0.0);
    for (int i = 0; i < nf; i++) lam[F[i]] = lf[i];
    // fixed dofs: x*_C = x0_C
    for (int i = 0; i < N; i++) {
        if (is_free[i]) continue;
        double hl = 0;
        for (int j = 0; j < N; j++) hl += H[(size_t)i * N + j] * lam[j];
        out.pose[i] += xbar[i] - hl;
    }
    // - (1/m) E_xs^T w at pose xe, added to out with a scale
    auto add_exs = [&](const double* xe, const std::vector<double>& w, double scale) {
        for (int b = 0; b < nb; b++) {
            if (pre[b].type != 2) continue;
            double g24[24];
            std::vector<double> h24(576);
            body_energy_state_derivs(pre[b], xe + 6 * b, p.gravity, h, g24, h24.data());
            for (int j = 6; j < 24; j++) {
                double acc = 0;
                for (int i = 0; i < 6; i++) acc += w[6 * b + i] * h24[24 * i + j];
                acc *= scale;
                if (j < 12) out.pose[6 * b + j - 6] += acc;
                else if (j < 15) out.vel[6 * b + j - 12] += acc;
                else out.Qdot[9 * b + j - 15] += acc;
            }
        }
    };
    add_exs(x, lam, -1.0 / M);

    // the initial stiffness
    if (rec.dkappa_dk0 != 0) {
        double kbar = 0;
        for (int i = 0; i < N; i++) kbar += lam[i] * gBx[i];
        kbar *= -rec.dkappa_dk0 / M;
        if (kbar != 0) {
            std::vector<double> x0(N);
            for (int b = 0; b < nb; b++)
                for (int k = 0; k < 6; k++) x0[6 * b + k] = pre[b].pose_t0[k];
            std::vector<double> gE(N, 0.0), gB, HE((size_t)N * N, 0.0), HB((size_t)N * N, 0.0);
            for (int b = 0; b < nb; b++) {
                if (pre[b].type != 2) continue;
                double g6[6], h36[36];
                body_energy(pre[b], &x0[6 * b], p.gravity, h, g6, h36);
                for (int r = 0; r < 6; r++) {
                    gE[6 * b + r] = g6[r];
                    for (int c = 0; c < 6; c++) HE[(size_t)(6 * b + r) * N + 6 * b + c] = h36[6 * r + c];
                }
            }
            BSR hb;
            std::vector<Constraint> cs = pr.constraints(x0.data());
            barrier_term(s, x0.data(), cs, p.dhat, p.dmin, gB, hb, false);
            Problem::add_bsr(hb, N, 1.0, HB);
            double gg = 0, ge = 0;
            for (int k = 0; k < N; k++) {
                gg += gB[k] * gB[k];
                ge += gB[k] * gE[k];
            }
            const double k0 = -ge / gg;
            const double sc = -kbar / gg;
            for (int i = 0; i < N; i++) {
                double u = 0;
                for (int j = 0; j < N; j++)
                    u += HB[(size_t)i * N + j] * (gE[j] + 2 * k0 * gB[j]) + HE[(size_t)i * N + j] * gB[j];
                out.pose[i] += sc * u;
            }
            add_exs(x0.data(), gB, sc);
        }
    }
    return true;
}

} // namespace orc

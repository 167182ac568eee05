// Per-body inertial energy with its gradient and 6x6 Hessian.
//
// Replaces compute_energy_term / compute_body_energy with the default
// implicit Euler integration (src/problems/distance_barrier_rb_problem.cpp:
// 706-944): for a dynamic body with pose x = (q, theta), Q = R(theta),
//   E = 1/2 m q.q - m q.(q0 + h (v0 + h g))              (unless q is fixed)
//     + 1/2 tr(Q J Q^T) - tr(Q J (Q0 + h Qdot0)^T)        (unless theta is fixed)
// with J = diag(1/2 (-I0 + I1 + I2), ...) from the principal moments
// (compute_J, :253-259).  The rotational derivatives use dQ/dtheta and
// d2Q/dtheta2 from the closed-form body frame (rotation.cuh).  The position
// block of the Hessian is m I (already positive definite; the reference's
// project_to_psd at :767-768 leaves it unchanged).
#include "common.cuh"
#include "rotation.cuh"
#include "sort.cuh"

namespace rigc {

__global__ void k_body_energy(const double* __restrict__ x, const int* __restrict__ type, int nb,
                              rigc_body_state s, double g0, double g1, double g2, double h,
                              double* __restrict__ energy, double* __restrict__ grad,
                              double* __restrict__ hess)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    double e = 0, g[6] = { 0, 0, 0, 0, 0, 0 }, H[36];
    for (int k = 0; k < 36; k++) H[k] = 0;
    if (type[b] == RIGC_BODY_DYNAMIC) {
        const int fixed = s.dof_fixed[b];
        const double m = s.mass[b];
        const double* q = x + 6 * b;
        const double* q0 = s.x_t0 + 6 * b;
        const double* v0 = s.v_t0 + 6 * b;
        const double grav[3] = { g0, g1, g2 };
        if ((fixed & 7) != 7) {
            double qq = 0, qh = 0;
            for (int i = 0; i < 3; i++) {
                double hat = q0[i] + h * (v0[i] + h * grav[i]);
                qq += q[i] * q[i];
                qh += q[i] * hat;
                g[i] = m * q[i] - m * hat;
                H[7 * i] = m;
            }
            e += 0.5 * m * qq - m * qh;
        }
        if ((fixed & 56) != 56) {
            const double* I = s.moment + 3 * b;
            double J[3] = { 0.5 * (-I[0] + I[1] + I[2]), 0.5 * (I[0] - I[1] + I[2]),
                            0.5 * (I[0] + I[1] - I[2]) };
            double t[3] = { q[3], q[4], q[5] };
            double F[kFrameDoubles];
            body_frame(t, F);
            double t0[3] = { q0[3], q0[4], q0[5] };
            double Q0[9];
            rot_rn(t0, Q0);
            const double* Qd = s.Qdot_t0 + 9 * b;
            // D = Q - T, T = Q0 + h Qdot0; E = sum_ik J_k (1/2 Q_ik^2 - Q_ik T_ik)
            double D[9];
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) {
                    double T = Q0[3 * i + k] + h * Qd[3 * i + k];
                    double Qv = F[3 * i + k];
                    e += J[k] * (0.5 * Qv * Qv - Qv * T);
                    D[3 * i + k] = Qv - T;
                }
            for (int a = 0; a < 3; a++) {
                const double* dA = F + 9 + 9 * a;
                double acc = 0;
                for (int i = 0; i < 3; i++)
                    for (int k = 0; k < 3; k++) acc += J[k] * dA[3 * i + k] * D[3 * i + k];
                g[3 + a] = acc;
                for (int c = a; c < 3; c++) {
                    const double* dC = F + 9 + 9 * c;
                    const double* d2 = F + 36 + 9 * sym_index(a, c);
                    double hh = 0;
                    for (int i = 0; i < 3; i++)
                        for (int k = 0; k < 3; k++)
                            hh += J[k] * (d2[3 * i + k] * D[3 * i + k] + dA[3 * i + k] * dC[3 * i + k]);
                    H[6 * (3 + a) + 3 + c] = hh;
                    H[6 * (3 + c) + 3 + a] = hh;
                }
            }
        }
    }
    energy[b] = e;
    if (grad)
        for (int k = 0; k < 6; k++) grad[6 * b + k] = g[k];
    if (hess)
        for (int k = 0; k < 36; k++) hess[36 * (size_t)b + k] = H[k];
}

int body_energy(Ctx& c, const rigc_body_state& s, const double* x, const double gravity[3],
                double h, double* energy_host, double* grad, double* hess)
{
    const int nb = c.s.nb;
    cudaStream_t st = c.stream;
    RIGC_TRY(c.scratch[0].reserve((size_t)(nb + 1) * sizeof(double)));
    double* e = c.scratch[0].as<double>();
    RIGC_COUNT_LAUNCH();
    k_body_energy<<<grid_for(nb, 128), 128, 0, st>>>(x, c.s.type, nb, s, gravity[0], gravity[1],
                                                     gravity[2], h, e, grad, hess);
    RIGC_CUDA(cudaGetLastError());
    double* e_dev = reinterpret_cast<double*>(c.d_scalars.as<char>() + 2560);
    RIGC_TRY(sum_f64(e, nb, e_dev, c.scratch[1], st));
    RIGC_CUDA(cudaMemcpyAsync(c.h_scalars + 8, e_dev, sizeof(double), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    *energy_host = c.h_scalars[8];
    return RIGC_OK;
}

} // namespace rigc

// C ABI of the rigc library (declared in include/rigc.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>

#include "common.cuh"

namespace rigc {

int detect_candidates(Ctx& c, const double* x0, const double* x1, bool continuous, double infl);
int construct_constraints(Ctx& c, const double* x, double dhat, double dmin);
int launch_barrier_local(Ctx& c, const double* x, double dhat, double dmin, int flags,
                         double* energy, double* grad, double* blocks, double* hess);
int assemble_barrier(Ctx& c, bool with_hess);
int scene_sums(Ctx& c, const double* val, const int* bodies, int64_t n, const int64_t seg[4],
               std::vector<double>& out);
int run_ccd(Ctx& c, const double* x0, const double* x1, double toi_tol, int flags,
            double* toi_host, double* per);
int run_pl_ccd(Ctx& c, const double* x0, const double* x1, double dmin, double* toi_host, double* per);
int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf);
int sum_f64(const double* in, int64_t n, double* out_dev, DevBuf& tmp, cudaStream_t stream);
int body_energy(Ctx& c, const rigc_body_state& s, const double* x, const double gravity[3],
                double h, double* energy_host, double* grad, double* hess);
int friction_setup(Ctx& c, const double* x0, double dhat, double kappa, double mu, double dmin);
int launch_friction_local(Ctx& c, const double* x, double epsvh, int flags, double* energy,
                          double* grad, double* blocks, double* hess);
int friction_term(Ctx& c, const double* x, double epsvh, int flags, rigc_barrier_out* out);
int sim_init(Ctx& c, const rigc_sim_params& p, const rigc_sim_state& s);
int sim_step(Ctx& c, rigc_step_stats* stats);
int sim_get_state(Ctx& c, double* poses, double* velocities, double* Qdot, double* kappa);
int sim_rollout(Ctx& c, int steps, int every, rigc_step_stats* stats);
int sim_scene_params(Ctx& c, const double* average_mass, const double* bbox_diagonal);
int sim_set_kinematic(Ctx& c, int body, double max_time, int64_t num_poses, const double* poses);
int autotune(Ctx& c, const double* x0, const double* x1, double dhat, double dmin,
             rigc_tune_report* rep);
int sim_backward(Ctx& c, const double* dp, const double* dv, const double* dq, double* gp,
                 double* gv, double* gq);
void sim_release(Ctx& c);

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches { 0 };

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

// broad phase, then record the candidate counts (also on an early exit)
int detect_and_count(Ctx& c, const double* x0, const double* x1, bool continuous,
                     double infl)
{
    int st = detect_candidates(c, x0, x1, continuous, infl);
    c.stats.cand_ee = c.cand.num_ee;
    c.stats.cand_fv = c.cand.num_fv;
    return st;
}

int barrier_term_impl(Ctx& c, const double* x, double dhat, double dmin, int flags,
                      rigc_barrier_out* out)
{
    const int64_t n = c.cons.num;
    const bool g = (flags & (RIGC_GRAD | RIGC_HESS)) != 0, h = (flags & RIGC_HESS) != 0;
    RIGC_TRY(c.c_energy.reserve((size_t)n * 8 + 8));
    if (g) RIGC_TRY(c.c_grad.reserve((size_t)n * 96 + 8));
    if (h) RIGC_TRY(c.c_blocks.reserve((size_t)n * 144 * 8 + 8));
    RIGC_TRY(launch_barrier_local(c, x, dhat, dmin, flags, c.c_energy.as<double>(),
                                  g ? c.c_grad.as<double>() : nullptr,
                                  h ? c.c_blocks.as<double>() : nullptr, nullptr));
    double* e_dev = reinterpret_cast<double*>(c.d_scalars.as<char>() + 2048);
    if (n > 0) {
        RIGC_TRY(sum_f64(c.c_energy.as<double>(), n, e_dev, c.scratch[6], c.stream));
    } else {
        RIGC_CUDA(cudaMemsetAsync(e_dev, 0, sizeof(double), c.stream));
    }
    if (g) {
        RIGC_TRY(assemble_barrier(c, h));
    }
    RIGC_CUDA(cudaMemcpyAsync(c.h_scalars, e_dev, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (h && n > 0)
        RIGC_CUDA(cudaMemcpyAsync(c.h_scalars + 1, c.d_scalars.as<int32_t>() + 1, sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    if (h && n > 0) {
        int32_t nn;
        std::memcpy(&nn, c.h_scalars + 1, sizeof(int32_t));
        c.nnzb = nn;
    }
    if (c.s.nscenes > 1) {
        const int64_t seg[4] = { 0, c.cons.num_vv, c.cons.num_vv + c.cons.num_ev,
                                 c.cons.num_vv + c.cons.num_ev + c.cons.num_ee };
        RIGC_TRY(scene_sums(c, c.c_energy.as<double>(), c.cons.bodies.as<int>(), n, seg,
                            c.h_scene_energy));
    } else {
        c.h_scene_energy.assign(1, c.h_scalars[0]);
    }
    if (out) {
        out->energy = c.h_scalars[0];
        out->nnzb = h ? c.nnzb : 0;
        out->grad = g ? c.grad.as<double>() : nullptr;
        out->row_ptr = h ? c.row_ptr.as<int32_t>() : nullptr;
        out->col = h ? c.col.as<int32_t>() : nullptr;
        out->val = h ? c.val.as<double>() : nullptr;
    }
    return RIGC_OK;
}

void set_error(int code, const char* what, const char* file, int line)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "rigc error %d: %s (%s:%d)", code, what, file, line);
    g_last_error = buf;
}

Ctx* ctx_of(rigc_ctx* c) { return reinterpret_cast<Ctx*>(c); }

template <class T> static int upload(T*& dst, const T* src, size_t n)
{
    if (n == 0) {
        dst = nullptr;
        return RIGC_OK;
    }
    RIGC_CUDA(cudaMalloc(&dst, n * sizeof(T)));
    RIGC_CUDA(cudaMemcpy(dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return RIGC_OK;
}

static void free_scene(Scene& s)
{
    void* ptrs[] = { s.rest, s.edges, s.faces, s.f2e, s.bvs, s.bes, s.bfs, s.group, s.grank,
                     s.type, s.rmax, s.vbody, s.ebody, s.fbody, s.edge_len, s.bscene,
                     s.scene_bstart };
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

static void release_all(Ctx* c)
{
    DevBuf* bufs[] = { &c->cand.ee, &c->cand.fv, &c->cons.type, &c->cons.verts, &c->cons.prims,
                       &c->cons.bodies, &c->cons.weight, &c->cons.eps, &c->frames, &c->c_energy,
                       &c->c_grad, &c->c_blocks, &c->grad, &c->row_ptr, &c->col, &c->val,
                       &c->d_scalars, &c->body_box, &c->body_in, &c->vbox, &c->ebox, &c->fbox,
                       &c->vin, &c->ein, &c->fin, &c->items_key, &c->items_val, &c->items_key2,
                       &c->items_val2, &c->seg, &c->pair_out, &c->pair_key, &c->large_list,
                       &c->x0_dev, &c->x1_dev, &c->rot_table, &c->cand_tol, &c->frame_keys, &c->ccd_pieces[0], &c->ccd_pieces[1], &c->ccd_pieces[2], &c->ccd_pieces[3], &c->pl_table,
                       &c->frame_vals, &c->fric.type, &c->fric.verts, &c->fric.bodies,
                       &c->fric.coef, &c->fric.v0c, &c->fric.V0, &c->fric.c_energy,
                       &c->fric.c_grad, &c->fric.c_blocks, &c->fric.grad, &c->fric.row_ptr,
                       &c->fric.col, &c->fric.val, &c->scene_toi, &c->scene_energy,
                       &c->bp_misc, &c->bp_deeper, &c->bp_sig, &c->bp_ec0,
                       &c->bp_eext, &c->bp_f32, &c->bp_cnt, &c->md_V, &c->md_rot,
                       &c->md_out, &c->isect.ee, &c->isect.fv };
    for (DevBuf* b : bufs) b->release();
    for (auto& b : c->scratch) b.release();
    sim_release(*c);
    if (c->h_scalars) cudaFreeHost(c->h_scalars);
    c->h_scalars = nullptr;
    free_scene(c->s);
}

} // namespace rigc

using namespace rigc;

extern "C" {

const char* rigc_status_string(int status)
{
    switch (status) {
    case RIGC_OK: return "ok";
    case RIGC_ERR_ARG: return "invalid argument";
    case RIGC_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case RIGC_ERR_OOM: return "device out of memory";
    case RIGC_ERR_QUEUE_OVERFLOW: return "CCD box stack overflow (conservative result)";
    case RIGC_ERR_ITER_LIMIT: return "CCD box budget exhausted (conservative result)";
    case RIGC_ERR_NAN: return "non-finite input";
    case RIGC_ERR_TOO_LARGE: return "input exceeds the entry point's fixed capacity";
    case RIGC_ERR_SOLVE: return "the Hessian of the free dofs could not be factorised";
    default: return "unknown status";
    }
}

static int ctx_create(const rigc_scene_desc* d, int num_scenes, const int32_t* body_scene,
                      rigc_ctx** out);

int rigc_ctx_create(const rigc_scene_desc* d, rigc_ctx** out)
{
    return ctx_create(d, 1, nullptr, out);
}

int rigc_ctx_create_batched(const rigc_scene_desc* d, int32_t num_scenes,
                            const int32_t* body_scene, rigc_ctx** out)
{
    if (!d || !out || num_scenes < 1 || (d->num_bodies > 0 && !body_scene)) return RIGC_ERR_ARG;
    for (int b = 0; b < d->num_bodies; b++)
        if (body_scene[b] < 0 || body_scene[b] >= num_scenes || (b && body_scene[b] < body_scene[b - 1]))
            return RIGC_ERR_ARG;
    return ctx_create(d, num_scenes, body_scene, out);
}

static int ctx_create(const rigc_scene_desc* d, int num_scenes, const int32_t* body_scene,
                      rigc_ctx** out)
{
    if (!d || !out) return RIGC_ERR_ARG;
    *out = nullptr;
    if (d->num_bodies < 0 || d->num_vertices < 0 || d->num_edges < 0 || d->num_faces < 0)
        return RIGC_ERR_ARG;
    if (d->num_bodies > 0 && (!d->body_vertex_start || !d->body_edge_start || !d->body_face_start
                              || !d->group_ids || !d->body_types || !d->r_max))
        return RIGC_ERR_ARG;
    if (d->num_vertices > 0 && !d->rest_vertices) return RIGC_ERR_ARG;
    if (d->num_edges > 0 && !d->edges) return RIGC_ERR_ARG;
    if (d->num_faces > 0 && (!d->faces || !d->faces_to_edges)) return RIGC_ERR_ARG;
    if ((int64_t)d->num_vertices >= (1ll << 30) || (int64_t)d->num_edges >= (1ll << 30)
        || (int64_t)d->num_faces >= (1ll << 30))
        return RIGC_ERR_ARG;
    const int nb = d->num_bodies, nv = d->num_vertices, ne = d->num_edges, nf = d->num_faces;
    // validate prefix arrays and indices on the host
    if (nb > 0) {
        if (d->body_vertex_start[0] != 0 || d->body_vertex_start[nb] != nv) return RIGC_ERR_ARG;
        if (d->body_edge_start[0] != 0 || d->body_edge_start[nb] != ne) return RIGC_ERR_ARG;
        if (d->body_face_start[0] != 0 || d->body_face_start[nb] != nf) return RIGC_ERR_ARG;
        for (int b = 0; b < nb; b++)
            if (d->body_vertex_start[b + 1] < d->body_vertex_start[b]
                || d->body_edge_start[b + 1] < d->body_edge_start[b]
                || d->body_face_start[b + 1] < d->body_face_start[b])
                return RIGC_ERR_ARG;
    }
    for (int i = 0; i < 2 * ne; i++)
        if (d->edges[i] < 0 || d->edges[i] >= nv) return RIGC_ERR_ARG;
    for (int i = 0; i < 3 * nf; i++) {
        if (d->faces[i] < 0 || d->faces[i] >= nv) return RIGC_ERR_ARG;
        if (d->faces_to_edges[i] < 0 || d->faces_to_edges[i] >= ne) return RIGC_ERR_ARG;
    }
    Ctx* c = new Ctx;
    Scene& s = c->s;
    s.nb = nb;
    s.nv = nv;
    s.ne = ne;
    s.nf = nf;
    s.avg_edge_len = d->average_edge_length;
    std::vector<int> vbody(nv), ebody(ne), fbody(nf);
    std::vector<double> elen(ne);
    for (int b = 0; b < nb; b++) {
        for (int i = d->body_vertex_start[b]; i < d->body_vertex_start[b + 1]; i++) vbody[i] = b;
        for (int i = d->body_edge_start[b]; i < d->body_edge_start[b + 1]; i++) ebody[i] = b;
        for (int i = d->body_face_start[b]; i < d->body_face_start[b + 1]; i++) fbody[i] = b;
        s.max_body_vertices = std::max(s.max_body_vertices,
                                       d->body_vertex_start[b + 1] - d->body_vertex_start[b]);
    }
    for (int e = 0; e < ne; e++) {
        const double* a = d->rest_vertices + 3 * d->edges[2 * e];
        const double* b = d->rest_vertices + 3 * d->edges[2 * e + 1];
        double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
        elen[e] = std::sqrt((d0 * d0 + d1 * d1) + d2 * d2);
    }
    s.h_bvs.assign(d->body_vertex_start, d->body_vertex_start + nb + 1);
    s.h_type.assign(d->body_types, d->body_types + nb);
    int st = RIGC_OK;
    auto chk = [&](int r) {
        if (st == RIGC_OK) st = r;
    };
    chk(upload(s.rest, d->rest_vertices, (size_t)3 * nv));
    chk(upload(s.edges, d->edges, (size_t)2 * ne));
    chk(upload(s.faces, d->faces, (size_t)3 * nf));
    chk(upload(s.f2e, d->faces_to_edges, (size_t)3 * nf));
    chk(upload(s.bvs, d->body_vertex_start, (size_t)nb + 1));
    chk(upload(s.bes, d->body_edge_start, (size_t)nb + 1));
    chk(upload(s.bfs, d->body_face_start, (size_t)nb + 1));
    chk(upload(s.group, d->group_ids, (size_t)nb));
    {
        // dense ranks of the group ids: the hash grid keys items by group
        std::vector<int> ids(d->group_ids, d->group_ids + nb);
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        std::vector<int> rank(nb);
        for (int b = 0; b < nb; b++)
            rank[b] = (int)(std::lower_bound(ids.begin(), ids.end(), d->group_ids[b]) - ids.begin());
        int bits = 1;
        while (bits < 31 && ((int64_t)1 << bits) < (int64_t)ids.size()) bits++;
        s.group_bits = bits;
        chk(upload(s.grank, rank.data(), (size_t)nb));
    }
    chk(upload(s.type, d->body_types, (size_t)nb));
    chk(upload(s.rmax, d->r_max, (size_t)nb));
    chk(upload(s.vbody, vbody.data(), (size_t)nv));
    chk(upload(s.ebody, ebody.data(), (size_t)ne));
    chk(upload(s.fbody, fbody.data(), (size_t)nf));
    chk(upload(s.edge_len, elen.data(), (size_t)ne));
    // scenes (one unless batched): scene of each body and first body of each
    std::vector<int> bscene(nb, 0), sstart(num_scenes + 1, nb);
    for (int b = nb - 1; b >= 0; b--) {
        bscene[b] = body_scene ? body_scene[b] : 0;
        sstart[bscene[b]] = b;
    }
    for (int k = num_scenes - 1; k >= 0; k--) sstart[k] = std::min(sstart[k], sstart[k + 1]);
    s.nscenes = num_scenes;
    s.h_scene_bstart = sstart;
    s.h_bes.assign(d->body_edge_start, d->body_edge_start + nb + 1);
    s.h_bfs.assign(d->body_face_start, d->body_face_start + nb + 1);
    chk(upload(s.bscene, bscene.data(), (size_t)nb));
    chk(upload(s.scene_bstart, sstart.data(), (size_t)num_scenes + 1));
    chk(c->d_scalars.reserve(4096));
    if (st == RIGC_OK) {
        cudaError_t e = cudaMallocHost(&c->h_scalars, 4096);
        if (e != cudaSuccess) st = RIGC_ERR_OOM;
    }
    if (st != RIGC_OK) {
        release_all(c);
        delete c;
        return st;
    }
    *out = reinterpret_cast<rigc_ctx*>(c);
    return RIGC_OK;
}

int rigc_ctx_destroy(rigc_ctx* ctx)
{
    if (!ctx) return RIGC_ERR_ARG;
    Ctx* c = ctx_of(ctx);
    cudaStreamSynchronize(c->stream);
    release_all(c);
    delete c;
    return RIGC_OK;
}

int rigc_set_stream(rigc_ctx* ctx, void* stream)
{
    if (!ctx) return RIGC_ERR_ARG;
    ctx_of(ctx)->stream = static_cast<cudaStream_t>(stream);
    return RIGC_OK;
}

int rigc_get_stats(const rigc_ctx* ctx, rigc_stats* out)
{
    if (!ctx || !out) return RIGC_ERR_ARG;
    *out = reinterpret_cast<const Ctx*>(ctx)->stats;
    out->kernel_launches = launch_count();
    return RIGC_OK;
}

int rigc_copy(rigc_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    if (!ctx || (bytes && (!dst || !src))) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    if (bytes) RIGC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

int rigc_world_vertices(rigc_ctx* ctx, const double* x, double* V)
{
    if (!ctx || !x || !V) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    return compute_world_vertices_rn(c, x, V, c.scratch[5]);
}

int rigc_detect_candidates(rigc_ctx* ctx, const double* x0, const double* x1, int continuous,
                           double inflation, rigc_candidates* out)
{
    if (!ctx || !x0 || (continuous && !x1) || !(inflation >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(detect_and_count(c, x0, x1, continuous != 0, inflation));
    if (out) {
        out->num_ee = c.cand.num_ee;
        out->num_fv = c.cand.num_fv;
        out->ee = c.cand.ee.as<int32_t>();
        out->fv = c.cand.fv.as<int32_t>();
    }
    return RIGC_OK;
}

int rigc_set_candidates(rigc_ctx* ctx, int64_t num_ee, const int32_t* ee, int64_t num_fv,
                        const int32_t* fv)
{
    if (!ctx || num_ee < 0 || num_fv < 0 || (num_ee && !ee) || (num_fv && !fv))
        return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    for (int64_t i = 0; i < 2 * num_ee; i++)
        if (ee[i] < 0 || ee[i] >= c.s.ne) return RIGC_ERR_ARG;
    for (int64_t i = 0; i < num_fv; i++)
        if (fv[2 * i] < 0 || fv[2 * i] >= c.s.nf || fv[2 * i + 1] < 0 || fv[2 * i + 1] >= c.s.nv)
            return RIGC_ERR_ARG;
    RIGC_TRY(c.cand.ee.reserve((size_t)num_ee * 8 + 8));
    RIGC_TRY(c.cand.fv.reserve((size_t)num_fv * 8 + 8));
    if (num_ee)
        RIGC_CUDA(cudaMemcpyAsync(c.cand.ee.ptr, ee, num_ee * 8, cudaMemcpyHostToDevice, c.stream));
    if (num_fv)
        RIGC_CUDA(cudaMemcpyAsync(c.cand.fv.ptr, fv, num_fv * 8, cudaMemcpyHostToDevice, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    c.cand.num_ee = num_ee;
    c.cand.num_fv = num_fv;
    c.stats.cand_ee = num_ee;
    c.stats.cand_fv = num_fv;
    return RIGC_OK;
}

int rigc_num_scenes(const rigc_ctx* ctx)
{
    return ctx ? reinterpret_cast<const Ctx*>(ctx)->s.nscenes : 0;
}

int rigc_scene_tois(rigc_ctx* ctx, double* toi_host)
{
    if (!ctx || !toi_host) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    for (int k = 0; k < c.s.nscenes; k++)
        toi_host[k] = k < (int)c.h_scene_toi.size() ? c.h_scene_toi[k] : INFINITY;
    return RIGC_OK;
}

int rigc_scene_barrier_energies(rigc_ctx* ctx, double* energy_host)
{
    if (!ctx || !energy_host) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    for (int k = 0; k < c.s.nscenes; k++)
        energy_host[k] = k < (int)c.h_scene_energy.size() ? c.h_scene_energy[k] : 0.0;
    return RIGC_OK;
}

int rigc_set_ccd_budget(rigc_ctx* ctx, int64_t max_boxes_per_candidate)
{
    if (!ctx || max_boxes_per_candidate < 1) return RIGC_ERR_ARG;
    ctx_of(ctx)->ccd_max_boxes = max_boxes_per_candidate;
    return RIGC_OK;
}

int rigc_earliest_toi(rigc_ctx* ctx, const double* x0, const double* x1, double toi_tol,
                      int flags, double* toi_host, double* per_candidate)
{
    if (!ctx || !x0 || !x1 || !toi_host || !(toi_tol > 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    // the poses may have changed since the candidates were found: no frames
    // are taken over from the broad phase
    c.bp_table.valid = false;
    return run_ccd(c, x0, x1, toi_tol, flags, toi_host, per_candidate);
}

int rigc_compute_earliest_toi(rigc_ctx* ctx, const double* x0, const double* x1, double dmin,
                              double* toi_host)
{
    if (!ctx || !x0 || !x1 || !toi_host || !(dmin >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(detect_and_count(c, x0, x1, true, dmin / 2.0));
    return run_ccd(c, x0, x1, 1e-4, 0, toi_host, nullptr);
}

int rigc_earliest_toi_piecewise_linear(rigc_ctx* ctx, const double* x0, const double* x1,
                                       double dmin, double* toi_host, double* per_candidate)
{
    if (!ctx || !x0 || !x1 || !toi_host || !(dmin >= 0)) return RIGC_ERR_ARG;
    return run_pl_ccd(*ctx_of(ctx), x0, x1, dmin, toi_host, per_candidate);
}

int rigc_set_pl_search(rigc_ctx* ctx, int32_t per_lane)
{
    if (!ctx || per_lane < -1 || per_lane > 1) return RIGC_ERR_ARG;
    ctx_of(ctx)->tune.pl_per_lane = per_lane;
    return RIGC_OK;
}

int rigc_set_ccd_window(rigc_ctx* ctx, int32_t window_log2)
{
    if (!ctx || window_log2 < -1 || window_log2 > 30) return RIGC_ERR_ARG;
    ctx_of(ctx)->tune.ccd_window_log2 = window_log2;
    return RIGC_OK;
}

int rigc_compute_earliest_toi_piecewise_linear(rigc_ctx* ctx, const double* x0, const double* x1,
                                               double dmin, double* toi_host)
{
    if (!ctx || !x0 || !x1 || !toi_host || !(dmin >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(detect_and_count(c, x0, x1, true, dmin / 2.0));
    c.bp_table.valid = false;
    return run_pl_ccd(c, x0, x1, dmin, toi_host, nullptr);
}

int rigc_construct_constraint_set(rigc_ctx* ctx, const double* x, double dhat, double dmin,
                                  rigc_constraints* out)
{
    if (!ctx || !x || !(dhat > 0) || !(dmin >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    if (c.s.nb <= 1) {
        c.cons.num = c.cons.num_vv = c.cons.num_ev = c.cons.num_ee = c.cons.num_fv = 0;
    } else {
        RIGC_TRY(detect_and_count(c, x, x, false, (dhat + dmin) / 2.0));
        RIGC_TRY(construct_constraints(c, x, dhat, dmin));
    }
    if (out) {
        Constraints& C = c.cons;
        out->num = C.num;
        out->num_vv = C.num_vv;
        out->num_ev = C.num_ev;
        out->num_ee = C.num_ee;
        out->num_fv = C.num_fv;
        out->type = C.type.as<int32_t>();
        out->verts = C.verts.as<int32_t>();
        out->prims = C.prims.as<int32_t>();
        out->bodies = C.bodies.as<int32_t>();
        out->weight = C.weight.as<double>();
        out->eps_x = C.eps.as<double>();
    }
    return RIGC_OK;
}

int rigc_set_constraints(rigc_ctx* ctx, int64_t num, const int32_t* type, const int32_t* verts,
                         const int32_t* prims, const int32_t* bodies, const double* weight,
                         const double* eps_x)
{
    if (!ctx || num < 0) return RIGC_ERR_ARG;
    if (num > 0 && (!type || !verts || !prims || !bodies || !weight || !eps_x)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    Constraints& C = c.cons;
    int64_t k[4] = { 0, 0, 0, 0 };
    for (int64_t i = 0; i < num; i++) {
        if (type[i] < 0 || type[i] > 3) return RIGC_ERR_ARG;
        int nvc = type[i] == 0 ? 2 : (type[i] == 1 ? 3 : 4);
        for (int j = 0; j < nvc; j++)
            if (verts[4 * i + j] < 0 || verts[4 * i + j] >= c.s.nv) return RIGC_ERR_ARG;
        for (int j = 0; j < 2; j++)
            if (bodies[2 * i + j] < 0 || bodies[2 * i + j] >= c.s.nb) return RIGC_ERR_ARG;
        k[type[i]]++;
    }
    RIGC_TRY(C.type.reserve((size_t)num * 4 + 8));
    RIGC_TRY(C.verts.reserve((size_t)num * 16 + 8));
    RIGC_TRY(C.prims.reserve((size_t)num * 8 + 8));
    RIGC_TRY(C.bodies.reserve((size_t)num * 8 + 8));
    RIGC_TRY(C.weight.reserve((size_t)num * 8 + 8));
    RIGC_TRY(C.eps.reserve((size_t)num * 8 + 8));
    cudaStream_t st = c.stream;
    if (num > 0) {
        RIGC_CUDA(cudaMemcpyAsync(C.type.ptr, type, num * 4, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(C.verts.ptr, verts, num * 16, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(C.prims.ptr, prims, num * 8, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(C.bodies.ptr, bodies, num * 8, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(C.weight.ptr, weight, num * 8, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(C.eps.ptr, eps_x, num * 8, cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaStreamSynchronize(st));
    }
    C.num = num;
    C.num_vv = k[0];
    C.num_ev = k[1];
    C.num_ee = k[2];
    C.num_fv = k[3];
    return RIGC_OK;
}

int rigc_barrier_term(rigc_ctx* ctx, const double* x, double dhat, double dmin, int flags,
                      rigc_barrier_out* out)
{
    if (!ctx || !x || !(dhat > 0) || !(dmin >= 0)) return RIGC_ERR_ARG;
    return barrier_term_impl(*ctx_of(ctx), x, dhat, dmin, flags, out);
}

int rigc_barrier_local_terms(rigc_ctx* ctx, const double* x, double dhat, double dmin, int flags,
                             double* energy, double* grad, double* hess)
{
    if (!ctx || !x || !(dhat > 0) || !(dmin >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(launch_barrier_local(c, x, dhat, dmin, flags, energy, grad, nullptr, hess));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

int rigc_body_energy(rigc_ctx* ctx, const rigc_body_state* state, const double* x,
                     const double gravity[3], double h, double* energy_host, double* grad,
                     double* hess)
{
    if (!ctx || !state || !x || !gravity || !energy_host || !(h > 0)) return RIGC_ERR_ARG;
    if (!state->mass || !state->moment || !state->x_t0 || !state->v_t0 || !state->Qdot_t0
        || !state->dof_fixed)
        return RIGC_ERR_ARG;
    return body_energy(*ctx_of(ctx), *state, x, gravity, h, energy_host, grad, hess);
}

int rigc_friction_setup(rigc_ctx* ctx, const double* x_t0, double dhat, double barrier_stiffness,
                        double coefficient_friction, int64_t* num_out)
{
    if (!ctx || !x_t0 || !(dhat > 0) || !(barrier_stiffness >= 0) || !(coefficient_friction >= 0))
        return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(friction_setup(c, x_t0, dhat, barrier_stiffness, coefficient_friction, 0.0));
    if (num_out) *num_out = c.fric.num;
    return RIGC_OK;
}

int rigc_get_friction(rigc_ctx* ctx, rigc_friction_view* out)
{
    if (!ctx || !out) return RIGC_ERR_ARG;
    Friction& F = ctx_of(ctx)->fric;
    out->num = F.num;
    out->mu = F.mu;
    out->type = F.type.as<int32_t>();
    out->verts = F.verts.as<int32_t>();
    out->bodies = F.bodies.as<int32_t>();
    out->coef = F.coef.as<double>();
    return RIGC_OK;
}

int rigc_friction_term(rigc_ctx* ctx, const double* x, double epsv_times_h, int flags,
                       rigc_barrier_out* out)
{
    if (!ctx || !x || !(epsv_times_h > 0)) return RIGC_ERR_ARG;
    return friction_term(*ctx_of(ctx), x, epsv_times_h, flags, out);
}

int rigc_friction_local_terms(rigc_ctx* ctx, const double* x, double epsv_times_h, int flags,
                              double* energy, double* grad, double* hess)
{
    if (!ctx || !x || !(epsv_times_h > 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(launch_friction_local(c, x, epsv_times_h, flags, energy, grad, nullptr, hess));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

int rigc_sim_init(rigc_ctx* ctx, const rigc_sim_params* params, const rigc_sim_state* state)
{
    if (!ctx || !params || !state || !state->mass || !state->moment || !state->dof_fixed
        || !state->poses || !state->velocities || !state->Qdot)
        return RIGC_ERR_ARG;
    const rigc_sim_params& p = *params;
    if (!(p.timestep > 0) || !(p.dhat > 0) || !(p.dmin >= 0) || !(p.average_mass > 0)
        || !(p.world_bbox_diagonal > 0) || p.max_newton_iterations < 1 || p.newton_polish < 0
        || !(p.ccd_rescale > 0 && p.ccd_rescale <= 1)
        || (p.trajectory_type != RIGC_TRAJECTORY_RIGID && p.trajectory_type != RIGC_TRAJECTORY_PIECEWISE_LINEAR))
        return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    // the batched step takes per-scene times of impact from the rigid CCD only
    if (c.s.nscenes > 1 && p.trajectory_type != RIGC_TRAJECTORY_RIGID) return RIGC_ERR_ARG;
    for (int i = 0; i < 6 * c.s.nb; i++)
        if (!std::isfinite(state->poses[i]) || !std::isfinite(state->velocities[i])) return RIGC_ERR_NAN;
    return sim_init(c, p, *state);
}

int rigc_sim_step(rigc_ctx* ctx, int32_t num_steps, rigc_step_stats* stats)
{
    if (!ctx || num_steps < 0) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    if (stats) *stats = rigc_step_stats {};
    for (int32_t k = 0; k < num_steps; k++) RIGC_TRY(sim_step(c, stats));
    return RIGC_OK;
}

int rigc_sim_get_state(rigc_ctx* ctx, double* poses, double* velocities, double* Qdot,
                       double* barrier_stiffness)
{
    if (!ctx) return RIGC_ERR_ARG;
    return sim_get_state(*ctx_of(ctx), poses, velocities, Qdot, barrier_stiffness);
}

int rigc_autotune(rigc_ctx* ctx, const double* x0, const double* x1, double dhat, double dmin,
                  rigc_tune_report* report)
{
    if (!ctx || !x0 || !x1 || !(dhat > 0) || !(dmin >= 0)) return RIGC_ERR_ARG;
    return autotune(*ctx_of(ctx), x0, x1, dhat, dmin, report);
}

int rigc_set_tune(rigc_ctx* ctx, int32_t ccd_blocks_per_sm, int32_t cache_slots_per_body,
                  int32_t barrier_per_warp, int32_t ccd_seeds_log2, int32_t ccd_hand_off,
                  int32_t ccd_warp)
{
    if (!ctx || ccd_blocks_per_sm < 0 || cache_slots_per_body < 0 || barrier_per_warp < 0
        || barrier_per_warp > 32 || cache_slots_per_body > (1 << 16) || ccd_seeds_log2 < -1
        || ccd_seeds_log2 > 5 || ccd_hand_off < -1 || ccd_warp < -1 || ccd_warp > 5)
        return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    c.tune.ccd_blocks_per_sm = ccd_blocks_per_sm;
    c.tune.cache_slots_per_body = cache_slots_per_body;
    c.tune.barrier_per_warp = barrier_per_warp;
    c.tune.ccd_seeds_log2 = ccd_seeds_log2;
    c.tune.ccd_hand_off = ccd_hand_off;
    c.tune.ccd_warp = ccd_warp;
    return RIGC_OK;
}

int rigc_sim_scene_params(rigc_ctx* ctx, const double* average_mass, const double* bbox_diagonal)
{
    if (!ctx) return RIGC_ERR_ARG;
    return sim_scene_params(*ctx_of(ctx), average_mass, bbox_diagonal);
}

int rigc_sim_set_kinematic(rigc_ctx* ctx, int32_t body, double max_time, int64_t num_poses,
                           const double* poses)
{
    if (!ctx) return RIGC_ERR_ARG;
    return sim_set_kinematic(*ctx_of(ctx), body, max_time, num_poses, poses);
}

int rigc_sim_rollout(rigc_ctx* ctx, int32_t num_steps, int32_t checkpoint_every,
                     rigc_step_stats* stats)
{
    if (!ctx || num_steps < 0 || checkpoint_every < 1) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    if (stats) *stats = rigc_step_stats {};
    return sim_rollout(c, num_steps, checkpoint_every, stats);
}

int rigc_sim_backward(rigc_ctx* ctx, const double* d_poses, const double* d_velocities,
                      const double* d_Qdot, double* g_poses, double* g_velocities, double* g_Qdot)
{
    if (!ctx) return RIGC_ERR_ARG;
    return sim_backward(*ctx_of(ctx), d_poses, d_velocities, d_Qdot, g_poses, g_velocities,
                        g_Qdot);
}

int rigc_narrow_phase_host(rigc_ctx* ctx, const double* x0_host, const double* x1_host,
                           double dhat, double dmin, double* toi_host, double* energy_host,
                           double* grad_host, int32_t* row_ptr_host, int32_t* col_host,
                           double* val_host, int64_t nnzb_cap, int64_t* nnzb_host)
{
    if (!ctx || !x0_host || !x1_host || !toi_host || !energy_host || !grad_host || !row_ptr_host
        || !nnzb_host || !(dhat > 0) || !(dmin >= 0) || nnzb_cap < 0)
        return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    const size_t xb = (size_t)6 * c.s.nb * sizeof(double);
    for (size_t i = 0; i < 6 * (size_t)c.s.nb; i++)
        if (!std::isfinite(x0_host[i]) || !std::isfinite(x1_host[i])) return RIGC_ERR_NAN;
    RIGC_TRY(c.x0_dev.reserve(xb + 8));
    RIGC_TRY(c.x1_dev.reserve(xb + 8));
    cudaStream_t st = c.stream;
    RIGC_CUDA(cudaMemcpyAsync(c.x0_dev.ptr, x0_host, xb, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(c.x1_dev.ptr, x1_host, xb, cudaMemcpyHostToDevice, st));
    const double* x0 = c.x0_dev.as<double>();
    const double* x1 = c.x1_dev.as<double>();
    int st_toi = rigc_compute_earliest_toi(ctx, x0, x1, dmin, toi_host);
    if (st_toi != RIGC_OK && st_toi != RIGC_ERR_QUEUE_OVERFLOW && st_toi != RIGC_ERR_ITER_LIMIT)
        return st_toi;
    RIGC_TRY(rigc_construct_constraint_set(ctx, x0, dhat, dmin, nullptr));
    rigc_barrier_out bo;
    RIGC_TRY(barrier_term_impl(c, x0, dhat, dmin, RIGC_GRAD | RIGC_HESS | RIGC_PROJECT_PSD, &bo));
    *energy_host = bo.energy;
    *nnzb_host = bo.nnzb;
    RIGC_CUDA(cudaMemcpyAsync(grad_host, bo.grad, xb, cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(row_ptr_host, bo.row_ptr, (size_t)(c.s.nb + 1) * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, st));
    if (bo.nnzb > 0 && bo.nnzb <= nnzb_cap && col_host && val_host) {
        RIGC_CUDA(cudaMemcpyAsync(col_host, bo.col, (size_t)bo.nnzb * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaMemcpyAsync(val_host, bo.val, (size_t)bo.nnzb * 36 * sizeof(double),
                                  cudaMemcpyDeviceToHost, st));
    }
    RIGC_CUDA(cudaStreamSynchronize(st));
    return st_toi;
}

} // extern "C"

// Constraint-set construction on the device.
//
// Replaces ipc::construct_constraint_set as DistanceBarrierConstraint::
// construct_constraint_set calls it (src/opt/distance_barrier_constraint.cpp:
// 267-306, V_rest = V): for every discrete EE / FV candidate, classify the
// closest features, keep the pair when the squared distance is below
// (dhat + dmin)^2, turn it into a VV, EV, EE (mollified when
// |ea x eb|^2 < 1e-3 |ea|^2 |eb|^2) or FV constraint, and merge duplicate VV / EV
// constraints into one with a multiplicity.  Duplicates are merged by a sort
// on the constraint key; the output is ordered vv | ev | ee | fv, each by key.
#include "common.cuh"
#include "geometry_rn.cuh"
#include "sort.cuh"

namespace rigc {

// per-body R (9) and p (3), exact round-to-nearest evaluation
__global__ void k_body_rot_rn(const double* __restrict__ x, int nb, double* __restrict__ out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    double t[3] = { x[6 * b + 3], x[6 * b + 4], x[6 * b + 5] };
    double R[9];
    rot_rn(t, R);
    for (int i = 0; i < 9; i++) out[12 * b + i] = R[i];
    out[12 * b + 9] = x[6 * b];
    out[12 * b + 10] = x[6 * b + 1];
    out[12 * b + 11] = x[6 * b + 2];
}

__global__ void k_world_vertices_rn(const double* __restrict__ rest, const int* __restrict__ vbody,
                                    int nv, const double* __restrict__ rot,
                                    double* __restrict__ V)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const double* f = rot + 12 * vbody[i];
    double R[9], p[3], v[3], o[3];
    for (int k = 0; k < 9; k++) R[k] = f[k];
    for (int k = 0; k < 3; k++) {
        p[k] = f[9 + k];
        v[k] = rest[3 * (size_t)i + k];
    }
    world_vertex_rn(R, p, v, o);
    V[3 * (size_t)i] = o[0];
    V[3 * (size_t)i + 1] = o[1];
    V[3 * (size_t)i + 2] = o[2];
}

int body_rot_rn(Ctx& c, const double* x, double* out)
{
    RIGC_COUNT_LAUNCH();
    k_body_rot_rn<<<grid_for(c.s.nb, 128), 128, 0, c.stream>>>(x, c.s.nb, out);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf)
{
    RIGC_TRY(rotbuf.reserve((size_t)12 * c.s.nb * sizeof(double)));
    RIGC_COUNT_LAUNCH();
    k_body_rot_rn<<<grid_for(c.s.nb, 128), 128, 0, c.stream>>>(x, c.s.nb, rotbuf.as<double>());
    RIGC_COUNT_LAUNCH();
    k_world_vertices_rn<<<grid_for(c.s.nv, 256), 256, 0, c.stream>>>(
        c.s.rest, c.s.vbody, c.s.nv, rotbuf.as<double>(), V);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// raw record of an active candidate
struct Raw {
    int kind;      // 0 VV, 1 EV, 2 EE, 3 FV
    int v[4];
    int p0, p1;    // key primitives
    double eps;
};

__device__ __forceinline__ bool classify(int64_t i, int64_t nee, const int2* __restrict__ ee,
                                         const int2* __restrict__ fv, const int* __restrict__ E,
                                         const int* __restrict__ F, const int* __restrict__ F2E,
                                         const double* __restrict__ V, double off, Raw& r)
{
    auto P = [&](int k) { return V + 3 * (size_t)k; };
    if (i < nee) {
        int ea = ee[i].x, eb = ee[i].y;
        int a0 = E[2 * ea], a1 = E[2 * ea + 1], b0 = E[2 * eb], b1 = E[2 * eb + 1];
        int t = ee_type_rn(P(a0), P(a1), P(b0), P(b1));
        double d;
        switch (t) {
        case EE_EA0_EB0: d = pp_sqdist_rn(P(a0), P(b0)); break;
        case EE_EA0_EB1: d = pp_sqdist_rn(P(a0), P(b1)); break;
        case EE_EA1_EB0: d = pp_sqdist_rn(P(a1), P(b0)); break;
        case EE_EA1_EB1: d = pp_sqdist_rn(P(a1), P(b1)); break;
        case EE_EA_EB0: d = pl_sqdist_rn(P(b0), P(a0), P(a1)); break;
        case EE_EA_EB1: d = pl_sqdist_rn(P(b1), P(a0), P(a1)); break;
        case EE_EA0_EB: d = pl_sqdist_rn(P(a0), P(b0), P(b1)); break;
        case EE_EA1_EB: d = pl_sqdist_rn(P(a1), P(b0), P(b1)); break;
        default: d = ll_sqdist_rn(P(a0), P(a1), P(b0), P(b1)); break;
        }
        if (!(d < off)) return false;
        double ua[3], ub[3];
        sub3_rn(P(a0), P(a1), ua);
        sub3_rn(P(b0), P(b1), ub);
        double eps_x = RMUL(RMUL(1e-3, dot3_rn(ua, ua)), dot3_rn(ub, ub));
        if (ee_cross_sqnorm_rn(P(a0), P(a1), P(b0), P(b1)) < eps_x) t = EE_EA_EB;
        r.eps = 0;
        r.v[2] = r.v[3] = -1;
        auto vv = [&](int x, int y) {
            r.kind = 0;
            r.v[0] = min(x, y);
            r.v[1] = max(x, y);
            r.p0 = r.v[0];
            r.p1 = r.v[1];
        };
        auto ev = [&](int e, int v) {
            r.kind = 1;
            r.v[0] = v;
            r.v[1] = E[2 * e];
            r.v[2] = E[2 * e + 1];
            r.p0 = e;
            r.p1 = v;
        };
        switch (t) {
        case EE_EA0_EB0: vv(a0, b0); break;
        case EE_EA0_EB1: vv(a0, b1); break;
        case EE_EA1_EB0: vv(a1, b0); break;
        case EE_EA1_EB1: vv(a1, b1); break;
        case EE_EA_EB0: ev(ea, b0); break;
        case EE_EA_EB1: ev(ea, b1); break;
        case EE_EA0_EB: ev(eb, a0); break;
        case EE_EA1_EB: ev(eb, a1); break;
        default:
            r.kind = 2;
            r.v[0] = a0; r.v[1] = a1; r.v[2] = b0; r.v[3] = b1;
            r.p0 = ea;
            r.p1 = eb;
            r.eps = eps_x;
        }
        return true;
    }
    int64_t k = i - nee;
    int f = fv[k].x, v = fv[k].y;
    int f0 = F[3 * f], f1 = F[3 * f + 1], f2 = F[3 * f + 2];
    int t = pt_type_rn(P(v), P(f0), P(f1), P(f2));
    double d;
    switch (t) {
    case PT_P_T0: d = pp_sqdist_rn(P(v), P(f0)); break;
    case PT_P_T1: d = pp_sqdist_rn(P(v), P(f1)); break;
    case PT_P_T2: d = pp_sqdist_rn(P(v), P(f2)); break;
    case PT_P_E0: d = pl_sqdist_rn(P(v), P(f0), P(f1)); break;
    case PT_P_E1: d = pl_sqdist_rn(P(v), P(f1), P(f2)); break;
    case PT_P_E2: d = pl_sqdist_rn(P(v), P(f2), P(f0)); break;
    default: d = ptplane_sqdist_rn(P(v), P(f0), P(f1), P(f2)); break;
    }
    if (!(d < off)) return false;
    r.eps = 0;
    r.v[2] = r.v[3] = -1;
    auto vv = [&](int x, int y) {
        r.kind = 0;
        r.v[0] = min(x, y);
        r.v[1] = max(x, y);
        r.p0 = r.v[0];
        r.p1 = r.v[1];
    };
    auto ev = [&](int e) {
        r.kind = 1;
        r.v[0] = v;
        r.v[1] = E[2 * e];
        r.v[2] = E[2 * e + 1];
        r.p0 = e;
        r.p1 = v;
    };
    switch (t) {
    case PT_P_T0: vv(v, f0); break;
    case PT_P_T1: vv(v, f1); break;
    case PT_P_T2: vv(v, f2); break;
    case PT_P_E0: ev(F2E[3 * f]); break;
    case PT_P_E1: ev(F2E[3 * f + 1]); break;
    case PT_P_E2: ev(F2E[3 * f + 2]); break;
    default:
        r.kind = 3;
        r.v[0] = v; r.v[1] = f0; r.v[2] = f1; r.v[3] = f2;
        r.p0 = f;
        r.p1 = v;
    }
    return true;
}

__global__ void k_classify_count(int64_t n, int64_t nee, const int2* __restrict__ ee,
                                 const int2* __restrict__ fv, const int* __restrict__ E,
                                 const int* __restrict__ F, const int* __restrict__ F2E,
                                 const double* __restrict__ V, double off,
                                 int32_t* __restrict__ flag)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Raw r;
    flag[i] = classify(i, nee, ee, fv, E, F, F2E, V, off, r) ? 1 : 0;
}

// key = kind (2 bits) | p0 (30 bits) | p1 (30 bits)
__global__ void k_classify_write(int64_t n, int64_t nee, const int2* __restrict__ ee,
                                 const int2* __restrict__ fv, const int* __restrict__ E,
                                 const int* __restrict__ F, const int* __restrict__ F2E,
                                 const double* __restrict__ V, double off,
                                 const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                                 uint64_t* __restrict__ keys, uint32_t* __restrict__ idx,
                                 int4* __restrict__ rverts, double* __restrict__ reps)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    Raw r;
    classify(i, nee, ee, fv, E, F, F2E, V, off, r);
    int32_t o = pos[i];
    keys[o] = ((uint64_t)r.kind << 60) | ((uint64_t)(uint32_t)r.p0 << 30) | (uint64_t)(uint32_t)r.p1;
    idx[o] = (uint32_t)o;
    rverts[o] = make_int4(r.v[0], r.v[1], r.v[2], r.v[3]);
    reps[o] = r.eps;
}

__global__ void k_cons_heads(const uint64_t* __restrict__ keys, int64_t m, int32_t* __restrict__ head)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_cons_emit(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ idx,
                            const int4* __restrict__ rverts, const double* __restrict__ reps,
                            const int32_t* __restrict__ head, const int32_t* __restrict__ segid,
                            int64_t m, const int* __restrict__ vbody, const int* __restrict__ ebody,
                            const int* __restrict__ fbody, int* __restrict__ type,
                            int4* __restrict__ verts, int2* __restrict__ prims,
                            int2* __restrict__ bodies, double* __restrict__ weight,
                            double* __restrict__ eps, int32_t* __restrict__ kind_count)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !head[i]) return;
    int64_t j = i + 1;
    while (j < m && !head[j]) j++;
    uint64_t k = keys[i];
    int kind = (int)(k >> 60);
    int p0 = (int)((k >> 30) & 0x3fffffffull), p1 = (int)(k & 0x3fffffffull);
    int s = segid[i];
    int4 rv = rverts[idx[i]];
    type[s] = kind;
    verts[s] = rv;
    prims[s] = make_int2(p0, p1);
    int b0, b1;
    switch (kind) {
    case 0: b0 = vbody[rv.x]; b1 = vbody[rv.y]; break;
    case 1: b0 = vbody[p1]; b1 = ebody[p0]; break;
    case 2: b0 = ebody[p0]; b1 = ebody[p1]; break;
    default: b0 = vbody[p1]; b1 = fbody[p0]; break;
    }
    bodies[s] = make_int2(b0, b1);
    weight[s] = (double)(j - i);
    eps[s] = reps[idx[i]];
    atomicAdd(&kind_count[kind], 1);
}

int construct_constraints(Ctx& c, const double* x, double dhat, double dmin)
{
    cudaStream_t st = c.stream;
    const int64_t nee = c.cand.num_ee, nfv = c.cand.num_fv, n = nee + nfv;
    DevBuf* S = c.scratch;
    // exact world vertices
    RIGC_TRY(S[4].reserve((size_t)3 * c.s.nv * sizeof(double)));
    double* V = S[4].as<double>();
    RIGC_TRY(compute_world_vertices_rn(c, x, V, S[5]));
    const double off = (dhat + dmin) * (dhat + dmin);
    c.cons.num = c.cons.num_vv = c.cons.num_ev = c.cons.num_ee = c.cons.num_fv = 0;
    if (n == 0) return RIGC_OK;
    RIGC_TRY(S[6].reserve((size_t)(2 * n + 16) * sizeof(int32_t)));
    int32_t* flag = S[6].as<int32_t>();
    int32_t* pos = flag + n;
    int32_t* cnt_dev = c.d_scalars.as<int32_t>();
    RIGC_COUNT_LAUNCH();
    k_classify_count<<<grid_for(n, 128), 128, 0, st>>>(
        n, nee, c.cand.ee.as<int2>(), c.cand.fv.as<int2>(), c.s.edges, c.s.faces, c.s.f2e, V, off,
        flag);
    RIGC_TRY(exclusive_scan_i32(flag, pos, n, cnt_dev, S[7], st));
    int32_t m;
    RIGC_CUDA(cudaMemcpyAsync(&m, cnt_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    if (m == 0) return RIGC_OK;
    // raw records
    RIGC_TRY(S[0].reserve((size_t)m * 8));
    RIGC_TRY(S[1].reserve((size_t)m * 4));
    RIGC_TRY(S[2].reserve((size_t)m * 8));
    RIGC_TRY(S[3].reserve((size_t)m * 4));
    DevBuf& rv = c.items_key2;
    DevBuf& re = c.items_val2;
    RIGC_TRY(rv.reserve((size_t)m * sizeof(int4)));
    RIGC_TRY(re.reserve((size_t)m * sizeof(double)));
    RIGC_COUNT_LAUNCH();
    k_classify_write<<<grid_for(n, 128), 128, 0, st>>>(
        n, nee, c.cand.ee.as<int2>(), c.cand.fv.as<int2>(), c.s.edges, c.s.faces, c.s.f2e, V, off,
        flag, pos, S[0].as<uint64_t>(), S[1].as<uint32_t>(), rv.as<int4>(), re.as<double>());
    RIGC_TRY(radix_sort_pairs<uint64_t>(S[0].as<uint64_t>(), S[1].as<uint32_t>(),
                                        S[2].as<uint64_t>(), S[3].as<uint32_t>(), m, 62,
                                        c.items_key, c.items_val, S[7], st));
    RIGC_TRY(S[6].reserve((size_t)(2 * m + 16) * sizeof(int32_t)));
    int32_t* head = S[6].as<int32_t>();
    int32_t* segid = head + m;
    RIGC_COUNT_LAUNCH();
    k_cons_heads<<<grid_for(m, 256), 256, 0, st>>>(S[2].as<uint64_t>(), m, head);
    RIGC_TRY(exclusive_scan_i32(head, segid, m, cnt_dev, S[7], st));
    int32_t nc;
    RIGC_CUDA(cudaMemcpyAsync(&nc, cnt_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    Constraints& C = c.cons;
    RIGC_TRY(C.type.reserve((size_t)nc * 4));
    RIGC_TRY(C.verts.reserve((size_t)nc * 16));
    RIGC_TRY(C.prims.reserve((size_t)nc * 8));
    RIGC_TRY(C.bodies.reserve((size_t)nc * 8));
    RIGC_TRY(C.weight.reserve((size_t)nc * 8));
    RIGC_TRY(C.eps.reserve((size_t)nc * 8));
    int32_t* kc = cnt_dev + 4;
    RIGC_CUDA(cudaMemsetAsync(kc, 0, 4 * sizeof(int32_t), st));
    RIGC_COUNT_LAUNCH();
    k_cons_emit<<<grid_for(m, 256), 256, 0, st>>>(
        S[2].as<uint64_t>(), S[3].as<uint32_t>(), rv.as<int4>(), re.as<double>(), head, segid, m,
        c.s.vbody, c.s.ebody, c.s.fbody, C.type.as<int>(), C.verts.as<int4>(), C.prims.as<int2>(),
        C.bodies.as<int2>(), C.weight.as<double>(), C.eps.as<double>(), kc);
    int32_t kinds[4];
    RIGC_CUDA(cudaMemcpyAsync(kinds, kc, sizeof(kinds), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    C.num = nc;
    C.num_vv = kinds[0];
    C.num_ev = kinds[1];
    C.num_ee = kinds[2];
    C.num_fv = kinds[3];
    return RIGC_OK;
}

} // namespace rigc

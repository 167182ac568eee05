// End-of-step intersection check.
//
// Replaces RigidBodyProblem::detect_intersections
// (src/physics/rigid_body_problem.cpp:289-360), 3D branch: the edge-face
// intersection candidates of the bodies at the given poses
// (detect_intersection_candidates_rigid_bvh, src/ccd/rigid/broad_phase.cpp:
// 265-302: close bodies with no inflation, element boxes of the vertex
// positions) and a segment-triangle test on each.  The candidates come from
// the hash grid of broad_phase.cu in its edge-face mode: every (edge, face)
// pair of different groups whose boxes overlap, a superset of the pairs that
// can intersect, so the answer does not depend on how the pairs are found.
//
// The segment-triangle test (ipc-toolkit's is_edge_intersecting_triangle is
// not in the reference tree; this is the orientation-based test of the
// computational-geometry literature): with orient(a, b, c, d) the signed
// volume det[b - a, c - a, d - a], the segment e0 e1 crosses the triangle
// t0 t1 t2 when e0 and e1 are not strictly on the same side of its plane
// (and not both on it: coplanar pairs count as not crossing), and the line
// e0 e1 passes inside the triangle: orient(e0, e1, t0, t1),
// orient(e0, e1, t1, t2), orient(e0, e1, t2, t0) all >= 0 or all <= 0.
// Everything is round-to-nearest double in a fixed order, the same as the
// oracle's, so both give the same answer on the same world vertices.
#include "common.cuh"
#include "rotation.cuh"

namespace rigc {

int detect_pairs(Ctx& c, const double* x0, const double* x1, bool continuous, double infl, int kind,
                 Candidates& out);
int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf);

__device__ __forceinline__ int orient_sign(const double* a, const double* b, const double* c,
                                           const double* d)
{
    const double u0 = RSUB(b[0], a[0]), u1 = RSUB(b[1], a[1]), u2 = RSUB(b[2], a[2]);
    const double v0 = RSUB(c[0], a[0]), v1 = RSUB(c[1], a[1]), v2 = RSUB(c[2], a[2]);
    const double w0 = RSUB(d[0], a[0]), w1 = RSUB(d[1], a[1]), w2 = RSUB(d[2], a[2]);
    const double c0 = RSUB(RMUL(v1, w2), RMUL(v2, w1));
    const double c1 = RSUB(RMUL(v2, w0), RMUL(v0, w2));
    const double c2 = RSUB(RMUL(v0, w1), RMUL(v1, w0));
    const double det = RADD(RADD(RMUL(u0, c0), RMUL(u1, c1)), RMUL(u2, c2));
    return det > 0 ? 1 : (det < 0 ? -1 : 0);
}

__device__ __forceinline__ bool edge_crosses_triangle(const double* e0, const double* e1,
                                                      const double* t0, const double* t1,
                                                      const double* t2)
{
    const int s0 = orient_sign(t0, t1, t2, e0), s1 = orient_sign(t0, t1, t2, e1);
    if (s0 == s1) return false;  // strictly on one side, or coplanar
    const int a = orient_sign(e0, e1, t0, t1), b = orient_sign(e0, e1, t1, t2),
              c = orient_sign(e0, e1, t2, t0);
    return (a >= 0 && b >= 0 && c >= 0) || (a <= 0 && b <= 0 && c <= 0);
}

// one thread per (face, edge) candidate; counts the crossing pairs
__global__ void k_edge_face_intersect(const int2* __restrict__ fe, int64_t n, const int* __restrict__ E,
                                      const int* __restrict__ F, const double* __restrict__ V,
                                      unsigned long long* __restrict__ count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool hit = false;
    if (i < n) {
        const int f = fe[i].x, e = fe[i].y;
        const double* e0 = V + 3 * (size_t)E[2 * e];
        const double* e1 = V + 3 * (size_t)E[2 * e + 1];
        const double* t0 = V + 3 * (size_t)F[3 * f];
        const double* t1 = V + 3 * (size_t)F[3 * f + 1];
        const double* t2 = V + 3 * (size_t)F[3 * f + 2];
        hit = edge_crosses_triangle(e0, e1, t0, t1, t2);
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

} // namespace rigc

extern "C" int rigc_detect_intersections(rigc_ctx* ctx, const double* x, int64_t* num_crossings)
{
    using namespace rigc;
    if (!ctx || !x || !num_crossings) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    *num_crossings = 0;
    if (c.s.nb <= 1) return RIGC_OK;
    RIGC_TRY(detect_pairs(c, x, x, false, 0.0, 1, c.isect));
    const int64_t n = c.isect.num_fv;
    if (n == 0) return RIGC_OK;
    RIGC_TRY(c.md_V.reserve((size_t)3 * c.s.nv * sizeof(double) + 8));
    RIGC_TRY(c.md_out.reserve(sizeof(unsigned long long)));
    RIGC_TRY(compute_world_vertices_rn(c, x, c.md_V.as<double>(), c.md_rot));
    unsigned long long* cnt = c.md_out.as<unsigned long long>();
    RIGC_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c.stream));
    RIGC_COUNT_LAUNCH();
    k_edge_face_intersect<<<grid_for(n, 256), 256, 0, c.stream>>>(
        c.isect.fv.as<int2>(), n, c.s.edges, c.s.faces, c.md_V.as<double>(), cnt);
    RIGC_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    RIGC_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    *num_crossings = (int64_t)h;
    return RIGC_OK;
}

// Shared definitions of the rigc CUDA library: context, device buffers,
// error handling and small device helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/rigc.h"

namespace rigc {

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

// CCD frame table: per body, interval frames (R as 9 intervals, p as 3) over
// the dyadic time nodes [k 2^-d, (k + 1) 2^-d] of depth d < 7 (slot
// 2^d - 1 + k) and over [0, toi_tol] (slot 127)
constexpr int kRotTableSlots = 128;
// the rigid CCD's time tolerance of the line searches (the reference's 1e-4)
constexpr double kDefaultToiTol = 1e-4;
constexpr int kRotTableEntry = 24;

// ---------------------------------------------------------------------------
// error handling: every host function returns an int status; CUDA failures
// are recorded in the context and surface as RIGC_ERR_CUDA / RIGC_ERR_OOM.

struct Status {
    int code = RIGC_OK;
    std::string msg;
};

#define RIGC_CUDA(expr)                                                       \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) {                                              \
            ::rigc::set_error(_e == cudaErrorMemoryAllocation ? RIGC_ERR_OOM  \
                                                             : RIGC_ERR_CUDA, \
                              cudaGetErrorString(_e), __FILE__, __LINE__);    \
            return _e == cudaErrorMemoryAllocation ? RIGC_ERR_OOM             \
                                                   : RIGC_ERR_CUDA;           \
        }                                                                     \
    } while (0)

#define RIGC_TRY(expr)                                                        \
    do {                                                                      \
        int _s = (expr);                                                      \
        if (_s != RIGC_OK) return _s;                                         \
    } while (0)

void set_error(int code, const char* what, const char* file, int line);

// number of kernels this library has launched (for measurement)
void count_launch();
// kernels run by graph launches (counted after they ran)
void count_launches(int64_t n);
int64_t launch_count();
#define RIGC_COUNT_LAUNCH() ::rigc::count_launch()

// grow-only device buffer
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    int reserve(size_t n)
    {
        if (n <= bytes) return RIGC_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t want = n + n / 4 + 256;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e != cudaSuccess) {
            set_error(RIGC_ERR_OOM, cudaGetErrorString(e), __FILE__, __LINE__);
            return RIGC_ERR_OOM;
        }
        bytes = want;
        return RIGC_OK;
    }
    template <class T> T* as() const { return static_cast<T*>(ptr); }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

// ---------------------------------------------------------------------------
// context

struct Scene {
    int nb = 0, nv = 0, ne = 0, nf = 0;
    double avg_edge_len = 0;
    // device arrays
    double* rest = nullptr;        // nv x 3
    int* edges = nullptr;          // ne x 2
    int* faces = nullptr;          // nf x 3
    int* f2e = nullptr;            // nf x 3
    int* bvs = nullptr;            // nb + 1
    int* bes = nullptr;
    int* bfs = nullptr;
    int* group = nullptr;          // nb
    int* grank = nullptr;          // nb: rank of the body's group among the distinct group ids
    int group_bits = 1;            // bits of the largest rank
    int* type = nullptr;           // nb
    double* rmax = nullptr;        // nb
    int* vbody = nullptr;          // nv
    int* ebody = nullptr;          // ne
    int* fbody = nullptr;          // nf
    double* edge_len = nullptr;    // ne
    // host copies of the prefix arrays
    std::vector<int> h_bvs, h_type;
    int max_body_vertices = 0;
    // batched contexts: independent scenes, bodies ordered by scene
    int nscenes = 1;
    int* bscene = nullptr;         // nb, scene of each body
    int* scene_bstart = nullptr;   // nscenes + 1, first body of each scene
    std::vector<int> h_scene_bstart, h_bes, h_bfs;
};

struct Candidates {
    int64_t num_ee = 0, num_fv = 0;
    DevBuf ee, fv;  // int2
};

struct Constraints {
    int64_t num = 0, num_vv = 0, num_ev = 0, num_ee = 0, num_fv = 0;
    DevBuf type, verts, prims, bodies, weight, eps;
};

// lagged friction constraints (a copy of the collision constraints at the
// start of the step with their normal forces, closest points and bases) and
// the friction term's outputs
struct Friction {
    int64_t num = 0;
    double mu = 0;
    DevBuf type, verts, bodies, coef, v0c, V0;
    DevBuf c_energy, c_grad, c_blocks;
    DevBuf grad, row_ptr, col, val;
    int64_t nnzb = 0;
};

struct Sim;  // time-stepping state (step.cu)

struct Ctx {
    Scene s;
    cudaStream_t stream = 0;
    Candidates cand;
    Constraints cons;
    rigc_stats stats {};
    // barrier outputs
    DevBuf frames;        // per body rotation frame (R, dR, d2R)
    DevBuf c_energy, c_grad, c_blocks;
    DevBuf grad, row_ptr, col, val;
    int64_t nnzb = 0;
    // scratch
    DevBuf scratch[8];
    DevBuf host_pinned_dummy;
    DevBuf d_scalars;     // small device scalars (reductions, counters)
    double* h_scalars = nullptr;  // pinned host mirror
    // broad-phase buffers
    DevBuf body_box, body_in, vbox, ebox, fbox, vin, ein, fin;
    DevBuf items_key, items_val, items_key2, items_val2, seg, pair_out, pair_key;
    DevBuf large_list;
    // hash grid: call state, deeper-bisection flags,
    // cell filter, per-element cell ranges, float boxes, item counts
    DevBuf bp_misc, bp_deeper, bp_sig, bp_ec0, bp_eext, bp_f32, bp_cnt;
    int64_t bp_pair_hint[2] = { 0, 0 };  // largest EE / FV pair counts seen
    // The continuous broad phase leaves the interval frames of the included
    // bodies over the dyadic time nodes of depth < 7 and over [0, toi_tol]
    // in rot_table (the CCD's layout); the CCD right after it on the same
    // poses reuses them.
    struct {
        const double* x0 = nullptr;
        const double* x1 = nullptr;
        double toi_tol = 0;
        bool valid = false;
    } bp_table;
    // rigc_min_distance / rigc_detect_intersections: world vertices, their
    // rotation frames, the result; the edge-face intersection candidates
    DevBuf md_V, md_rot, md_out;
    Candidates isect;
    // temporary pose buffers for host entry points
    DevBuf x0_dev, x1_dev;
    // CCD: body frames over the top dyadic time intervals
    DevBuf rot_table;
    DevBuf cand_tol;  // CCD: per-candidate tolerances
    DevBuf frame_keys, frame_vals;  // CCD frame cache (hash table)
    DevBuf pl_table;  // piecewise-linear CCD: per-body piece frames and point rotations
    DevBuf ccd_pieces[4];           // CCD search pieces: a launch's input and output, the later windows' (two)
    Friction fric;
    int64_t ccd_max_boxes = int64_t(1) << 22;  // per-candidate CCD box budget
    // launch shapes chosen by rigc_autotune (0: the built-in choice)
    struct Tune {
        int ccd_blocks_per_sm = 0;     // resident k_ccd blocks per SM (0: occupancy limit)
        int cache_slots_per_body = 0;  // CCD frame-cache slots per body (0: 1024)
        int barrier_per_warp = 0;      // constraints per warp of k_barrier_local (0: by count)
        int ccd_seeds_log2 = -1;       // CCD searches per candidate, log2 (-1: by count)
        int ccd_hand_off = -1;         // CCD boxes per search piece before a hand-off (-1: default, 0: never)
        int ccd_window_log2 = -1;      // CCD first time window 2^-k (-1: built-in, 0: no windows)
        int ccd_warp = -1;             // CCD search per lane (0) or per warp (1); -1: by candidate count
        int pl_per_lane = -1;          // piecewise-linear CCD: a candidate per lane (1) or per warp (0, -1)
    } tune;
    Sim* sim = nullptr;
    // batched contexts: per-scene results of the last calls
    DevBuf scene_toi, scene_energy;
    // batched time step: scenes whose bodies enter the broad phase (device,
    // one int per scene; null: all)
    const int* scene_on = nullptr;
    std::vector<double> h_scene_toi, h_scene_energy;
};

Ctx* ctx_of(rigc_ctx* c);

// ---------------------------------------------------------------------------
// launch helpers

inline unsigned grid_for(int64_t n, int block)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

} // namespace rigc

// Per-constraint barrier terms for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: a plugin running inside a host
// application that owns the device memory (its own pool or a fixed budget),
// or a latency-critical loop where an allocation would synchronise the
// device.  They cannot create a rigc_ctx, so this entry point takes every
// input and output as caller-owned device memory and keeps its only working
// memory -- the per-body rotation frames (R, dR/dtheta, d2R/dtheta2, p; 96
// doubles per body) -- in a file-scope device array of fixed capacity.
//
// Facts a caller relies on:
//  * capacity: kMaxBodies bodies (3 MiB); larger scenes get
//    RIGC_ERR_TOO_LARGE before any work is queued;
//  * the array lives on every GPU that loads the library until the process
//    exits;
//  * host code cannot use the array's name as a device address; the address
//    is looked up once per device with cudaGetSymbolAddress, with that device
//    current, on the first call there -- so make the first call before any
//    stream capture;
//  * every call shares the array and it keeps the last call's contents;
//    each call rewrites all frames it reads before reading them, and calls
//    that overlap on the GPU race, so serialise them on one stream;
//  * constraint indices are checked on the device against num_bodies and
//    num_vertices; a constraint with an index out of range gets NaN energy,
//    gradient and Hessian and reads nothing (a host-side check would need a
//    copy of the device arrays and a synchronisation);
//  * nothing here allocates: no cudaMalloc, cudaFree or allocating library
//    call.
#include <mutex>

#include "common.cuh"

namespace rigc {

constexpr int kMaxBodies = RIGC_NOALLOC_MAX_BODIES;
constexpr int kFrameStride = 96;  // doubles per body frame
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_frames[(size_t)kMaxBodies * kFrameStride];

int launch_barrier_local_raw(const double* rest, int64_t nv, int nb, const double* x, int64_t n,
                             const int* ctype, const int* cverts, const int* cbodies,
                             const double* cweight, const double* ceps, double dhat, double dmin,
                             int flags, double* frames, double* energy, double* grad,
                             double* hess, cudaStream_t stream);

// device address of the working array, looked up once per device
static int frames_address(double** out)
{
    static std::mutex mu;
    static double* addr[kMaxDevices] = {};
    int dev = 0;
    RIGC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return RIGC_ERR_ARG;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        RIGC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_frames));
        addr[dev] = static_cast<double*>(p);
    }
    *out = addr[dev];
    return RIGC_OK;
}

} // namespace rigc

extern "C" int rigc_barrier_local_terms_noalloc(
    const double* rest_vertices, int64_t num_vertices, int32_t num_bodies, const double* x,
    int64_t num_constraints,
    const int32_t* type, const int32_t* verts, const int32_t* bodies, const double* weight,
    const double* eps_x, double dhat, double dmin, int flags, double* energy, double* grad,
    double* hess, void* cuda_stream)
{
    using namespace rigc;
    if (num_bodies < 0 || num_vertices < 0 || num_constraints < 0 || !(dhat > 0) || !(dmin >= 0))
        return RIGC_ERR_ARG;
    if (num_bodies > kMaxBodies) {
        set_error(RIGC_ERR_TOO_LARGE, "num_bodies exceeds RIGC_NOALLOC_MAX_BODIES", __FILE__,
                  __LINE__);
        return RIGC_ERR_TOO_LARGE;
    }
    if (num_bodies > 0 && !x) return RIGC_ERR_ARG;
    if (num_constraints > 0
        && (!rest_vertices || !type || !verts || !bodies || !weight || !eps_x))
        return RIGC_ERR_ARG;
    if (num_bodies == 0) return num_constraints == 0 ? RIGC_OK : RIGC_ERR_ARG;
    double* frames = nullptr;
    RIGC_TRY(frames_address(&frames));
    // the constraint arrays are device memory the host cannot inspect without
    // a copy and a synchronisation: the kernel checks every type, vertex and
    // body index against these limits and gives an out-of-range constraint
    // NaN outputs instead of reading past an array
    return launch_barrier_local_raw(rest_vertices, num_vertices, num_bodies, x, num_constraints,
                                    type, verts,
                                    bodies, weight, eps_x, dhat, dmin, flags, frames, energy,
                                    grad, hess, static_cast<cudaStream_t>(cuda_stream));
}

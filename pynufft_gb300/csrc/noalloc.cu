// Exact (deterministic) gridding that allocates nothing.
//
// nufft_y2k_exact_static is a variant of the deterministic gridding path
// (nufft_y2k on a plan created with NUFFT_FLAG_DETERMINISTIC) for callers
// that must not allocate device memory at call time: applications that hand
// all GPU memory to their own pool up front (a cudaMalloc there can fail or
// fragment the pool), and latency-critical code that cannot afford
// cudaMalloc/cudaFree (cudaFree synchronises the whole device).  The regular
// path creates its 64-bit fixed-point accumulators lazily with cudaMalloc on
// first use; this one uses a fixed scratch array compiled into the library.
//
// The scratch is a file-scope __device__ array of NUFFT_STATIC_SCRATCH_CELLS
// grid cells (2 x 8 bytes each, i.e. 16 MiB) plus the scale reduction
// buffers; every GPU that loads the library holds it until the process
// exits.  Host code cannot use the array's name as a device address, so the
// address is looked up with cudaGetSymbolAddress on the first call made in
// each CUDA context (with that context's device current) and kept for that
// context; a new context on the device (after cudaDeviceReset, say) is seen
// by its id and looked up again.  Make the first call on a device before any
// stream capture.  All calls share the array and it keeps the last call's
// contents (it is cleared at the start of each call); calls whose work
// overlaps on the GPU -- on different streams, or from different host
// threads -- race on it.
#include "nufft_internal.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

namespace nufft {
int launch_y2k_exact_into(const nufft_plan_s* p, const float2* y, float2* grid,
                          unsigned long long* acc, double* scal, cudaStream_t s);
}

namespace {

constexpr size_t kCells = NUFFT_STATIC_SCRATCH_CELLS;
constexpr int kScal = nufft::kScaleSlots;   // sum|y|, scale and the per-block partials
static_assert(kScal >= 2 + nufft::kAbsSumParts, "scale buffer smaller than its partial sums");

static __device__ __align__(256) unsigned long long g_acc[2 * kCells];
static __device__ __align__(256) double g_scal[kScal];

constexpr int kMaxDevices = 64;
struct Scratch {
    unsigned long long ctx_id = 0;   // context the addresses belong to (0: none yet)
    unsigned long long* acc = nullptr;
    double* scal = nullptr;
};
std::mutex g_mu;
Scratch g_scratch[kMaxDevices];

// Id of the calling thread's current context (unique for the process's
// lifetime, so a re-created context gets a new one), through driver entry
// points fetched by the runtime (the library does not link libcuda).
// Returns 0 if it cannot be found.
unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device addresses of the scratch arrays in the current device's context
// (which must be the plan's device).
int scratch_for_current_device(int plan_device, unsigned long long** acc, double** scal) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        nufft::set_error("nufft_y2k_exact_static: no usable current CUDA device");
        return NUFFT_ECUDA;
    }
    if (dev != plan_device) {
        nufft::set_error("nufft_y2k_exact_static: the plan's device (" +
                         std::to_string(plan_device) + ") is not the current device (" +
                         std::to_string(dev) + ")");
        return NUFFT_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    Scratch& c = g_scratch[dev];
    const unsigned long long ctx = current_context_id();
    if (ctx == 0 || c.ctx_id != ctx) {
        void* a = nullptr;
        void* b = nullptr;
        e = cudaGetSymbolAddress(&a, g_acc);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&b, g_scal);
        if (e != cudaSuccess) {
            nufft::set_error(std::string("nufft_y2k_exact_static: cudaGetSymbolAddress: ") +
                             cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
        c.acc = static_cast<unsigned long long*>(a);
        c.scal = static_cast<double*>(b);
        // the lookup made the runtime's context current if none was; an
        // unknown id (0) means the next call looks the addresses up again
        c.ctx_id = current_context_id();
    }
    *acc = c.acc;
    *scal = c.scal;
    return NUFFT_OK;
}

}  // namespace

extern "C" int nufft_y2k_exact_static(nufft_plan_t p, const void* y, void* k, void* stream) {
    if (!p) {
        nufft::set_error("nufft_y2k_exact_static: plan is NULL");
        return NUFFT_EINVAL;
    }
    if (!p->d_perm) {
        nufft::set_error("nufft_y2k_exact_static: nufft_set_points has not been called");
        return NUFFT_ENOPOINTS;
    }
    if (!k || (!y && p->M > 0)) {
        nufft::set_error("nufft_y2k_exact_static: NULL data pointer");
        return NUFFT_EINVAL;
    }
    const size_t cells = (size_t)p->ninst * p->prodK * p->B;
    if (cells > kCells) {
        nufft::set_error("nufft_y2k_exact_static: grid of " + std::to_string(cells) +
                         " cells (instances x prod(Kd) x batch) exceeds the static scratch of " +
                         std::to_string(kCells) + " cells");
        return NUFFT_EINVAL;
    }
    unsigned long long* acc = nullptr;
    double* scal = nullptr;
    int st = scratch_for_current_device(p->device, &acc, &scal);
    if (st != NUFFT_OK) return st;
    return nufft::launch_y2k_exact_into(p, static_cast<const float2*>(y), static_cast<float2*>(k),
                                        acc, scal, reinterpret_cast<cudaStream_t>(stream));
}

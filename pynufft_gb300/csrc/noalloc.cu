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
// exits.  Its device address is looked up once per device with
// cudaGetSymbolAddress on the first call made while that device is current,
// so make that first call before any stream capture.  All calls share the
// array and it keeps the last call's contents (it is cleared at the start
// of each call); calls whose work overlaps on the GPU -- on different
// streams, or from different host threads -- race on it.
#include "nufft_internal.cuh"

#include <mutex>

namespace nufft {
int launch_y2k_exact_into(const nufft_plan_s* p, const float2* y, float2* grid,
                          unsigned long long* acc, double* scal, cudaStream_t s);
}

namespace {

constexpr size_t kCells = NUFFT_STATIC_SCRATCH_CELLS;
constexpr int kScal = 2 + 1024;   // scale, sum|y| and per-block partials

static __device__ __align__(256) unsigned long long g_acc[2 * kCells];
static __device__ __align__(256) double g_scal[kScal];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned long long* g_acc_ptr[kMaxDevices] = {};
double* g_scal_ptr[kMaxDevices] = {};

// Device addresses of the scratch arrays for the current device.
int scratch_for_current_device(unsigned long long** acc, double** scal) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        nufft::set_error("nufft_y2k_exact_static: no usable current CUDA device");
        return NUFFT_ECUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_acc_ptr[dev]) {
        void* a = nullptr;
        void* c = nullptr;
        e = cudaGetSymbolAddress(&a, g_acc);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&c, g_scal);
        if (e != cudaSuccess) {
            nufft::set_error(std::string("nufft_y2k_exact_static: cudaGetSymbolAddress: ") +
                             cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
        g_acc_ptr[dev] = static_cast<unsigned long long*>(a);
        g_scal_ptr[dev] = static_cast<double*>(c);
    }
    *acc = g_acc_ptr[dev];
    *scal = g_scal_ptr[dev];
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
    int st = scratch_for_current_device(&acc, &scal);
    if (st != NUFFT_OK) return st;
    return nufft::launch_y2k_exact_into(p, static_cast<const float2*>(y), static_cast<float2*>(k),
                                        acc, scal, reinterpret_cast<cudaStream_t>(stream));
}

// Internal definitions shared by the pynufft_gb300 CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pynufft_gb300.h"

#define NUFFT_MAXDIM 3
#define NUFFT_MAXJ 16
#define NUFFT_MAXL 14     // L = ceil(N/3) reaches 14 at N = 40
#define NUFFT_NALPHA 16   // coefficient array length (>= MAXL + 1)

namespace nufft {

// Exact gridding: per-block partial sums of |re y| + |im y| reduced before the
// fixed-point scale is fixed; the scale buffer holds [sum |y|, scale,
// partials...].
constexpr int kAbsSumParts = 1024;
constexpr int kScaleSlots = 2 + kAbsSumParts;

// Most points of one sub-problem of the gather list (interpolation from a
// shared tile, plans of 8 or more coils): a bin's tile is loaded once unless
// the bin holds more.
constexpr int kGatherSub = 512;

// Row gridding (plans of 8 or more coils): a sub-problem takes up to
// kRowGroup consecutive bins along the innermost axis (3D) and at most
// row_sub_cap points, so the tile's halo along that axis is shared.
constexpr int kRowGroup = 4;
// Row sub-problems hold at most kRowSub2 (2D) / kRowSub3 (3D) points, so
// that the row kernels stage their coefficients and samples (all coils of a
// lane group) in shared memory three blocks per SM (8 coils in 3D, 32 in
// 2D): 32-coil radial adjoint 0.219 ms with 256 points (two blocks) against
// 0.200 ms; 8-coil kooshball with 448 points 11.0 ms fast against 9.6 ms
// with 320.  Both modes use the same lists, so their plans hold the same
// tables (and the deterministic sums do not depend on the plan's mode).
constexpr int kRowSub2 = 192;
constexpr int kRowSub3 = 320;
inline int row_sub_cap(int ndim) { return ndim == 2 ? kRowSub2 : kRowSub3; }

void set_error(const std::string& msg);

// Plan-time numerics of one axis (plan_math.cpp).
struct AxisParams {
    int N = 0, J = 0, K = 0, L = 0;
    float alpha[NUFFT_NALPHA];
    std::vector<double> sn;  // N
    std::vector<double> T;   // J*J, row major
};
int axis_params(int N, int J, int K, AxisParams& ap);
int derive_axis(AxisParams& ap);  // sn and T from N, J, K, L, alpha

// Constants of one axis used by the per-point table kernel (points.cu).
struct AxisConst {
    double gam;          // 2 pi / K
    double inv_ratio;    // N / K
    double lin;          // gam * (N - 1) / 2
    double half_N;       // N / 2
    int K, J, L, N;
    double alpha[NUFFT_MAXL + 1];
    double T[NUFFT_MAXJ * NUFFT_MAXJ];
};

// Everything a gather/scatter kernel needs, passed by value.
struct Geom {
    int ndim;
    int B;                    // coils (batch), fastest axis of x/k/y
    int K[3], J[3], JP[3];    // grid size, neighbours, table stride (J rounded up to even)
    int bs[3], nb[3];         // bin shape and bins per axis
    int T[3];                 // scatter tile extent per axis = bs + J - 1
    int64_t prodK;            // cells per instance
    int64_t nbin_inst;        // bins per instance
    int64_t M;                // total points
    int ninst;
    const int64_t* inst_start;   // ninst+1 prefix of points per instance (device)
    const int* perm;             // sorted -> original point index
    const int* pos[3];           // first footprint index per axis, sorted order
    const float2* coef[3];       // conj(u) coefficients, sorted order, stride JP
    const float* wpt;            // per point prod_d max_j |coef|, sorted order
    const int4* sub;             // gridding sub-problems: (bin, start, count, inst)
    int64_t nsub;
    int maxsub;                  // most points in one sub-problem
    const int4* gsub;            // gather sub-problems (plans of 8+ coils): bins split
    int64_t ngsub;               //   only past kGatherSub points
    const int4* rsub;            // row-gridding sub-problems (plans of 8+ coils):
    int64_t nrsub;               //   runs of <= kRowGroup bins along the innermost
    int rgroup;                  //   axis (rgroup bins), <= row_sub_cap points
    int cm_il;                   // row gridding target: 0 coil-major, 1 coil-major
                                 // row-interleaved (see nufft_plan_s), 2 coil-fastest
    int kmethod;                 // k2y lane mapping (NUFFT_K2Y_*), resolved
    int ymethod;                 // y2k lane mapping (NUFFT_Y2K_*), resolved
    int* kerr;                   // device flag: a bounded wait ran out (nufft_plan_check)
};

// Padded shared-tile layout of the paired-thread kernels: tile cell
// (x, y, z) (z fastest; tile extents T) sits at word x*sx + y*sy + z.  The
// stride of the axis whose taps the two threads of a point split (x in 3D,
// y in 2D) is padded to 16 mod 32, so the two threads of a point always
// address words 16 banks apart; rows (sy) are even, so a row of complex64
// cells starts on a 16-byte boundary (bulk-copy destinations); n is the
// padded cell count.
struct TileStrides {
    int sy, sx, n;
};
__host__ __device__ inline int pad_to_16_mod_32(int v) { return v + ((16 - v % 32) + 32) % 32; }
__host__ __device__ inline TileStrides tile_strides(int ndim, const int* T) {
    TileStrides s{0, 0, T[0]};
    if (ndim == 2) {
        s.sy = pad_to_16_mod_32(T[1]);
        s.n = T[0] * s.sy;
    } else if (ndim == 3) {
        s.sy = (T[2] + 1) & ~1;
        s.sx = pad_to_16_mod_32(T[1] * s.sy);
        s.n = T[0] * s.sx;
    }
    return s;
}
// Bank buckets per bin used to order the points of a bin: 16 residues of the
// padded address in 2D/3D (a warp holds 16 points, each split over two
// threads 16 banks apart), 32 in 1D (a warp holds 32 points).
__host__ __device__ inline int bank_keys(int ndim) { return ndim == 1 ? 32 : 16; }

}  // namespace nufft

struct nufft_plan_s {
    int ndim = 0;
    int Nd[3] = {1, 1, 1}, Kd[3] = {1, 1, 1}, Jd[3] = {1, 1, 1};
    int B = 1, ninst = 1, flags = 0;
    int64_t prodN = 1, prodK = 1;
    nufft::AxisParams ax[3];
    int bs[3] = {0, 0, 0};
    int user_bs[3] = {0, 0, 0};
    int maxsub = 0, user_maxsub = 0;
    int k2y_method = 0, y2k_method = 0;   // 0 = default for the geometry
    int device = 0;
    int num_sms = 0;

    // device buffers owned by the plan
    float* d_snd = nullptr;           // per-axis scaling factors (float32), concatenated
    nufft::AxisConst* d_axc = nullptr;
    float2* d_grid = nullptr;         // ninst * prodK * B oversampled grid workspace
    // adjoint's own grid (one coil, one instance, fast gridding): zeroed on a
    // side stream while the forward runs, so the adjoint's gridding needs no
    // memset on its own path; ev_zero marks the zeroing done, ev_adj the
    // last adjoint's reads of it done
    float2* d_grid_adj = nullptr;
    cudaStream_t zs = nullptr;
    cudaEvent_t ev_zero = nullptr, ev_adj = nullptr;
    bool adj_zeroed = false, adj_used = false;
    float2* d_ybuf = nullptr;         // M * B sample workspace (selfadjoint, CG)
    float2* d_maps = nullptr;         // coil sensitivities Nd x B (nufft_set_sense)
    int* d_kerr = nullptr;            // device error flag written by bounded waits
    // optional CUDA-event timing of the k2y / y2k kernels (nufft_plan_kernel_timing):
    // every kperiod-th launch (0: off) is bracketed; events are created once
    // and reused; kused[w] of kev[w] hold the records (start, stop, ...) since
    // timing was enabled, kseen[w] counts the launches
    int kperiod = 0;
    std::vector<cudaEvent_t> kev[2];  // [0] k2y, [1] y2k
    size_t kused[2] = {0, 0};
    size_t kseen[2] = {0, 0};
    size_t ybuf_elems = 0;

    // point data (valid after nufft_set_points)
    int64_t M = 0;
    std::vector<int64_t> counts;
    int64_t* d_inst_start = nullptr;
    int* d_perm = nullptr;
    int* d_pos = nullptr;             // ndim * M
    float* d_wpt = nullptr;           // M per-point weight bound prod_d max_j |coef|
    float2* d_coef = nullptr;         // sum_d M * JP[d]
    int4* d_sub = nullptr;
    int64_t nsub = 0;
    int4* d_gsub = nullptr;           // gather sub-problems (B >= 8)
    int64_t ngsub = 0;
    int4* d_rsub = nullptr;           // row-gridding sub-problems (B >= 8)
    int64_t nrsub = 0;
    int rgroup = 1;                   // bins per row sub-problem along the innermost axis
    int64_t nbins_total = 0;
    float wmax = 0.f;                 // max over points of prod_d max_j |coef|

    // deterministic gridding
    unsigned long long* d_igrid = nullptr;  // 2 * ninst * prodK * B fixed-point accumulators
    double* d_dscal = nullptr;              // [0] = sum |y|, [1] = fixed-point scale

    // CG workspace
    float2* d_cg = nullptr;           // r, p, q, xk: 4 * ninst * prodK * B
    double* d_cgs = nullptr;          // device scalars
    double* d_part = nullptr;         // per-block partial sums
    int part_blocks = 0;
    cudaGraphExec_t cg_init_exec = nullptr;   // captured CG set-up (keyed by y, maxiter, tols)
    cudaGraphExec_t cg_iter_exec = nullptr;   // captured chunk of CG iterations
    const void* cg_y = nullptr;
    int cg_maxiter = -1, cg_chunk = 0;
    double cg_rtol = 0, cg_atol = 0;

    cufftHandle fft = 0;              // all axes, every coil / instance
    cufftHandle fft_slab = 0;         // (y[,z]) FFTs on the first Nd[0] slabs
    cufftHandle fft_x = 0;            // x-axis FFTs over all slabs
    bool fft_ok = false, fft_pruned = false;
    bool fft_cm_pruned = false;       // B > 1: per-system pruned plans on the coil-major copy
    void* d_fftwork = nullptr;        // shared cuFFT work area
    float2* d_padin = nullptr;        // pruned forward: zero-padded input, first Nd[0] slabs
    float2* d_slabout = nullptr;      // pruned forward: slab-FFT output, other slabs zero
    bool pfft = false;                // own pruned power-of-two FFT passes (pfft.cu)
    float2* d_pfft_tw = nullptr;      // per-axis, per-stage twiddle tables, concatenated
    int pfft_tw_off[3][4] = {};       // [axis][stage] offsets into d_pfft_tw
    // 2D / 3D plans of a multiple of 8 coils, one instance, Kd in {128, 160,
    // 192, 256, 320, 384, 512, 640}: the own coil-batched passes (cfft.cu) transform the
    // coil-fastest grid directly (d_cm holds their intermediate arrays), and
    // the row gridding writes the coil-fastest grid
    bool cfft = false;
    float2* d_cfft_tw = nullptr;      // exp(-2 pi i m / Kd[0]), then / Kd[1]
    float2* d_cm = nullptr;           // B > 1: coil-major copy of the grid for the FFTs
    // B > 1 with per-system pruned 3D plans: zero-kept padded inputs (the
    // first Nd[0] slabs of every system) and slab-FFT outputs (slabs past
    // Nd[0] stay zero), so the forward writes only the image corner
    float2* d_cmpad = nullptr;
    float2* d_cmslab = nullptr;
    // Plans of several coils and one instance (2D, 3D): the coil-major
    // spectra are interleaved along the first axis, first-axis slab n0 of
    // coil b at (n0 B + b) times the slab size (prod(Kd) / K0), so the first
    // Nd[0] slabs of every coil are one contiguous run and the inner-axes
    // FFTs (fft_rows) skip the zero slabs (forward) and the slabs the crop
    // drops (inverse); fft_cols transforms along the first axis (stride B
    // times the slab size).  The forward pads the image corner into d_il_pad
    // (Nd[0] B slabs, kept zero outside the corner), transforms its slabs
    // into d_il_z (slabs past Nd[0] kept zero), whose first axis transforms
    // into d_cm.
    bool cm_il = false;
    cufftHandle fft_rows = 0;
    cufftHandle fft_cols = 0;
    float2* d_il_pad = nullptr;
    float2* d_il_z = nullptr;
    size_t dev_bytes = 0;

    nufft::Geom geom() const;
};

namespace nufft {

// error helpers --------------------------------------------------------------
#define NUFFT_CUDA_TRY(expr)                                                         \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess) {                                                     \
            ::nufft::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));  \
            return (_e == cudaErrorMemoryAllocation) ? NUFFT_ENOMEM : NUFFT_ECUDA;   \
        }                                                                            \
    } while (0)

#define NUFFT_CUFFT_TRY(expr)                                                        \
    do {                                                                             \
        cufftResult _r = (expr);                                                     \
        if (_r != CUFFT_SUCCESS) {                                                   \
            ::nufft::set_error(std::string(#expr) + ": cufft error " +               \
                               std::to_string((int)_r));                             \
            return NUFFT_ECUFFT;                                                     \
        }                                                                            \
    } while (0)

#define NUFFT_TRY(expr)                   \
    do {                                  \
        int _s = (expr);                  \
        if (_s != NUFFT_OK) return _s;    \
    } while (0)

inline int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return NUFFT_ECUDA;
    }
    return NUFFT_OK;
}

// points.cu
int set_points(nufft_plan_s* p, const int64_t* counts, const double* om, int om_on_device,
               cudaStream_t s);
void free_points(nufft_plan_s* p);

// interp.cu
int launch_k2y(nufft_plan_s* p, const float2* grid, float2* y, cudaStream_t s);
bool kernel_time_start(nufft_plan_s* p, int which, cudaStream_t s);  // true: this launch is timed
void kernel_time_stop(nufft_plan_s* p, int which, cudaStream_t s, bool started);
void kernel_time_clear(nufft_plan_s* p);     // forget the records, keep the events
void kernel_time_destroy(nufft_plan_s* p);   // free the events
int launch_y2k(nufft_plan_s* p, const float2* y, float2* grid, cudaStream_t s,
               bool pre_zeroed = false);   // pre_zeroed: grid already zero (fast mode)
// coil-major gridding (plans of 8 or more coils, interp_cm.cuh): whether the
// plan's geometry has the row kernels, and y2k into the p->d_cm layout
bool cm_path(const nufft_plan_s* p);
int launch_y2k_cm(nufft_plan_s* p, const float2* y, float2* grid_cm, cudaStream_t s,
                  bool pre_zeroed = false);
// deterministic plans: the row gridding's exact sums left in p->d_igrid
// (scale in p->d_dscal), unrounded
int launch_y2k_cm_fixed(nufft_plan_s* p, const float2* y, cudaStream_t s);
// the y2k stage into a coil-fastest spectrum (the row kernels and one
// transpose for deterministic plans that have them, else launch_y2k)
int launch_y2k_grid(nufft_plan_s* p, const float2* y, float2* k, cudaStream_t s);

// fftstage.cu
int launch_scale(const nufft_plan_s* p, const float2* in, float2* out, cudaStream_t s);
int launch_pad(const nufft_plan_s* p, const float2* xx, float2* grid, bool apply_sn,
               int dom_axis, cudaStream_t s);
int launch_crop(const nufft_plan_s* p, const float2* grid, float2* xx, bool apply_sn,
                bool divide_sn, cudaStream_t s);
int fft_exec(nufft_plan_s* p, float2* grid, int direction, cudaStream_t s);
// dom_axis >= 0: the image is also multiplied by -i (n_a - N_a/2) along that
// axis (the trajectory derivative)
int forward_from_image(nufft_plan_s* p, const float2* xx, bool apply_sn, float2* k,
                       cudaStream_t s, int dom_axis = -1);
int image_from_spectrum_coils(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn,
                              bool divide_sn, cudaStream_t s);
// several coils, coil-major spectra in p->d_cm: image -> spectra / spectra -> image
int image_to_cm(nufft_plan_s* p, const float2* xx, bool apply_sn, cudaStream_t s,
                int dom_axis = -1);
int cm_to_image(nufft_plan_s* p, float2* xx, bool apply_sn, bool divide_sn, cudaStream_t s);
// the coil-major spectra in p->d_cm -> coil-fastest spectrum k (one transpose)
int cm_to_grid(const nufft_plan_s* p, float2* k, cudaStream_t s);
int launch_pad_sense(const nufft_plan_s* p, const float2* x, float2* grid, cudaStream_t s);
int launch_crop_sense(const nufft_plan_s* p, const float2* grid, float2* x, cudaStream_t s);
int fft_init(nufft_plan_s* p);
void fft_destroy(nufft_plan_s* p);
// k (Kd) -> image: inverse transform, crop, / prod(Kd), x sn or / sn (B == 1)
int image_from_spectrum(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn,
                        bool divide_sn, cudaStream_t s);

// pfft.cu: own pruned power-of-two FFT passes (B == 1, one instance)
bool pfft_eligible(const nufft_plan_s* p);
int pfft_init(nufft_plan_s* p);
void pfft_free(nufft_plan_s* p);
int pfft_forward(nufft_plan_s* p, const float2* x, bool apply_sn, float2* k, cudaStream_t s);
int pfft_inverse(nufft_plan_s* p, const float2* k, float2* x, bool apply_sn, bool divide_sn,
                 cudaStream_t s);

// cfft.cu: own coil-batched passes on coil-fastest layouts (2D, several coils)
bool cfft_eligible(const nufft_plan_s* p);
int cfft_init(nufft_plan_s* p);
void cfft_free(nufft_plan_s* p);
int cfft_forward(nufft_plan_s* p, const float2* xx, bool apply_sn, int dom_axis, float2* k,
                 cudaStream_t s);
int cfft_inverse(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn, bool divide_sn,
                 cudaStream_t s);
// the same from a deterministic gridding's 64-bit fixed-point sums (ig: 2 x
// prod(Kd) x B; dscal[1] their scale), rounded inside the first pass
int cfft_inverse_fixed(nufft_plan_s* p, const unsigned long long* ig, const double* dscal,
                       float2* xx, bool apply_sn, bool divide_sn, cudaStream_t s);

// cg.cu
int solve_cg(nufft_plan_s* p, const float2* y, float2* x, int maxiter, double rtol,
             double atol, int* iters_out, cudaStream_t s);
void free_cg(nufft_plan_s* p);

// tv.cu
int solve_l1tvols(nufft_plan_s* p, const float2* y, float2* x, int maxiter, double rho,
                  cudaStream_t s);

}  // namespace nufft

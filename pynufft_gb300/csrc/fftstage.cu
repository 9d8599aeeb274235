// Image-side stages around the oversampled FFT.
//
//   x2xx / xx2x  multiply by the separable real scaling factor sn
//                (_x2xx_cpu / _xx2x_cpu, nufft/_nufft_class_methods_cpu.py:224-230, 346-351)
//   xx2k         zero-pad Nd -> Kd into the top-left corner, then a forward
//                FFT (_xx2k_cpu :232-249, preindex_copy src/_helper/helper.py:830-881)
//   k2xx         inverse FFT (normalised by 1/prod(Kd) as numpy.fft.ifftn), then
//                crop the top-left Nd corner (_k2xx_cpu :316-329)
// forward fuses x2xx into the pad pass and adjoint fuses xx2x into the crop
// pass, so each direction touches the image once and the grid once outside
// cuFFT.  The FFTs are cuFFT C2C plans (complex64), batched over coils.
#include "nufft_internal.cuh"

#include <algorithm>

namespace nufft {

struct ImgGeom {
    int ndim, B;
    int il;           // coil-major spectra row-interleaved (2D, one instance)
    int N[3], K[3];
    int64_t prodN, prodK;
    int64_t n_img;    // ninst * prodN * B
    int64_t n_grid;   // ninst * prodK * B
    const float* sn[3];
};

static ImgGeom img_geom(const nufft_plan_s* p) {
    ImgGeom g{};
    g.ndim = p->ndim;
    g.B = p->B;
    g.il = p->cm_il ? 1 : 0;
    int off = 0;
    for (int d = 0; d < 3; ++d) {
        g.N[d] = p->Nd[d];
        g.K[d] = p->Kd[d];
        g.sn[d] = p->d_snd + off;
        if (d < p->ndim) off += p->Nd[d];
    }
    g.prodN = p->prodN;
    g.prodK = p->prodK;
    g.n_img = (int64_t)p->ninst * p->prodN * p->B;
    g.n_grid = (int64_t)p->ninst * p->prodK * p->B;
    return g;
}

__device__ __forceinline__ float sn_of(const ImgGeom& g, const int (&n)[3]) {
    float v = __ldg(g.sn[0] + n[0]);
    if (g.ndim > 1) v *= __ldg(g.sn[1] + n[1]);
    if (g.ndim > 2) v *= __ldg(g.sn[2] + n[2]);
    return v;
}

// Row-wise kernels: one block per row of the last axis (all other indices
// fixed per block), threads along the row, so index arithmetic is one
// division chain per block and the row's accesses are contiguous.
template <int DIM>
__device__ __forceinline__ void row_index(int64_t r64, int e0, int e1, int64_t& inst, int& n0,
                                          int& n1) {
    // r enumerates (inst, i0[, i1]) over the extents (e0[, e1]) of the
    // leading axes; rows number fewer than 2^31, so 32-bit unsigned division
    // suffices.  Scalars only: no local-memory copies of parameter arrays.
    unsigned r = (unsigned)r64;
    n0 = n1 = 0;
    if (DIM == 3) {
        const unsigned q = r / (unsigned)e1;
        n1 = (int)(r - q * (unsigned)e1);
        r = q;
    }
    if (DIM >= 2) {
        const unsigned q = r / (unsigned)e0;
        n0 = (int)(r - q * (unsigned)e0);
        r = q;
    }
    inst = r;
}

template <int DIM>
__device__ __forceinline__ float lead_sn(const float* sn0, const float* sn1, int n0, int n1) {
    float s = 1.f;
    if (DIM >= 2) s *= __ldg(sn0 + n0);
    if (DIM == 3) s *= __ldg(sn1 + n1);
    return s;
}

template <int DIM>
__global__ void scale_rows_kernel(ImgGeom g, const float2* __restrict__ in, float2* __restrict__ out,
                                  int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    const int L = g.N[DIM - 1];
    const int B = g.B;
    const float s_lead = lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]);
    const float* snl = g.sn[DIM - 1];
    const size_t base = (size_t)r * L * B;
    for (int e = threadIdx.x; e < L * B; e += blockDim.x) {
        const int k = (B == 1) ? e : e / B;
        const float sc = s_lead * __ldg(snl + k);
        const float2 v = __ldg(in + base + e);
        out[base + e] = make_float2(v.x * sc, v.y * sc);
    }
  }
}

// grid row = x row * (sn if apply_sn) * (-i (n_a - N_a/2) if dom_axis == a),
// zero outside the Nd corner
template <int DIM>
__global__ void pad_rows_kernel(ImgGeom g, const float2* __restrict__ xx, float2* __restrict__ grid,
                                int apply_sn, int dom_axis, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.K[0], g.K[1], inst, n[0], n[1]);
    bool inside = true;
#pragma unroll
    for (int d = 0; d < DIM - 1; ++d) inside = inside && (n[d] < g.N[d]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    float2* dst = grid + (size_t)r * KL * B;
    if (!inside) {
        for (int e = threadIdx.x; e < KL * B; e += blockDim.x) dst[e] = make_float2(0.f, 0.f);
        continue;
    }
    const float s_lead = apply_sn ? lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]) : 1.f;
    float a_lead = 0.f;
    if (DIM >= 2 && dom_axis == 0) a_lead = (float)n[0] - 0.5f * (float)g.N[0];
    if (DIM == 3 && dom_axis == 1) a_lead = (float)n[1] - 0.5f * (float)g.N[1];
    int64_t xrow = inst;
    if (DIM >= 2) xrow = xrow * g.N[0] + n[0];
    if (DIM == 3) xrow = xrow * g.N[1] + n[1];
    const float2* src = xx + (size_t)xrow * NL * B;
    for (int e = threadIdx.x; e < KL * B; e += blockDim.x) {
        const int k = (B == 1) ? e : e / B;
        float2 v = make_float2(0.f, 0.f);
        if (k < NL) {
            v = __ldg(src + e);
            if (apply_sn) {
                const float sc = s_lead * __ldg(g.sn[last] + k);
                v.x *= sc;
                v.y *= sc;
            }
            if (dom_axis >= 0) {
                const float a = (dom_axis == last) ? (float)k - 0.5f * (float)NL : a_lead;
                v = make_float2(a * v.y, -a * v.x);
            }
        }
        dst[e] = v;
    }
  }
}

// Nd corner only: grid row (inst, n0[, n1]) first N cells = x row (* sn);
// every other cell of `grid` is left as it is (zero in the plan's padded
// input buffer, which nothing else writes).  One coil.
template <int DIM>
__global__ void corner_rows_kernel(ImgGeom g, const float2* __restrict__ xx, float2* __restrict__ grid,
                                   int apply_sn, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    int64_t grow = inst;
    if (DIM >= 2) grow = grow * g.K[0] + n[0];
    if (DIM == 3) grow = grow * g.K[1] + n[1];
    const float2* src = xx + (size_t)r * NL;
    float2* dst = grid + (size_t)grow * KL;
    const float s_lead = apply_sn ? lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]) : 1.f;
    for (int k = threadIdx.x; k < NL; k += blockDim.x) {
        float2 v = __ldg(src + k);
        if (apply_sn) {
            const float sc = s_lead * __ldg(g.sn[last] + k);
            v.x *= sc;
            v.y *= sc;
        }
        dst[k] = v;
    }
  }
}

// x row = grid row (first N of the last axis) / prod(Kd) * (sn if apply_sn) / (sn if divide_sn)
template <int DIM>
__global__ void crop_rows_kernel(ImgGeom g, const float2* __restrict__ grid, float2* __restrict__ xx,
                                 int apply_sn, int divide_sn, float norm, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    const float s_lead = lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]);
    int64_t krow = inst;
#pragma unroll
    for (int d = 0; d < last; ++d) krow = krow * g.K[d] + n[d];
    const float2* src = grid + (size_t)krow * KL * B;
    float2* dst = xx + (size_t)r * NL * B;
    for (int e = threadIdx.x; e < NL * B; e += blockDim.x) {
        const int k = (B == 1) ? e : e / B;
        float2 v = __ldg(src + e);
        float sc = norm;
        const float snv = s_lead * __ldg(g.sn[last] + k);
        if (apply_sn) sc *= snv;
        v.x *= sc;
        v.y *= sc;
        if (divide_sn) {
            v.x /= snv;
            v.y /= snv;
        }
        dst[e] = v;
    }
  }
}

// Element (leading indices n0[, n1], last-axis index k) of coil b of
// instance inst in the coil-major spectra: system-contiguous, or interleaved
// along the first axis (one instance): slab n0 of coil b at (n0 B + b) times
// the slab size.
template <int DIM>
__device__ __forceinline__ size_t cm_at(const ImgGeom& g, int64_t inst, int b, int n0, int n1,
                                        int k) {
    constexpr int last = DIM - 1;
    const int KL = g.K[last];
    if (DIM == 1) return ((size_t)inst * g.B + b) * g.prodK + k;
    if (g.il) {
        size_t slab = (size_t)n0 * g.B + b;
        if (DIM == 3) slab = slab * g.K[1] + n1;
        return slab * KL + k;
    }
    size_t row = (size_t)n0;
    if (DIM == 3) row = row * g.K[1] + n1;
    return ((size_t)inst * g.B + b) * g.prodK + row * KL + k;
}

// Several coils, coil-major spectra.  The grid of system (instance, coil)
// = inst * B + b is one contiguous Kd block of `cm`.  Pad: one block per grid
// row (inst, leading indices) writes that row for every coil (zero outside
// the Nd corner), reading the coil-fastest image row once through L1.
template <int DIM>
__global__ void pad_cm_rows_kernel(ImgGeom g, const float2* __restrict__ xx, float2* __restrict__ cm,
                                   int apply_sn, int dom_axis, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.K[0], g.K[1], inst, n[0], n[1]);
    bool inside = true;
#pragma unroll
    for (int d = 0; d < DIM - 1; ++d) inside = inside && (n[d] < g.N[d]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    int64_t xrow = inst;
#pragma unroll
    for (int d = 0; d < last; ++d) xrow = xrow * g.N[d] + n[d];
    const float s_lead = (apply_sn && inside) ? lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]) : 1.f;
    float a_lead = 0.f;
    if (DIM >= 2 && dom_axis == 0) a_lead = (float)n[0] - 0.5f * (float)g.N[0];
    if (DIM == 3 && dom_axis == 1) a_lead = (float)n[1] - 0.5f * (float)g.N[1];
    const float2* src = xx + (size_t)xrow * NL * B;
    for (int e = threadIdx.x; e < KL * B; e += blockDim.x) {
        const int b = e / KL, k = e - b * KL;
        float2 v = make_float2(0.f, 0.f);
        if (inside && k < NL) {
            v = __ldg(src + (size_t)k * B + b);
            if (apply_sn) {
                const float sc = s_lead * __ldg(g.sn[last] + k);
                v.x *= sc;
                v.y *= sc;
            }
            if (dom_axis >= 0) {   // x -i (n_a - N_a/2): the trajectory derivative
                const float a = (dom_axis == last) ? (float)k - 0.5f * (float)NL : a_lead;
                v = make_float2(a * v.y, -a * v.x);
            }
        }
        cm[cm_at<DIM>(g, inst, b, n[0], n[1], k)] = v;
    }
  }
}

// Several coils, 3D: the Nd corner of every system's zero-kept padded input
// (its first N0 slabs, `slabsz` = N0 * K1 * K2 cells per system); one block
// per image row (inst, n0, n1) reads the coil-fastest row once and writes it
// for every coil.  Cells outside the corner are never written (zero).
__global__ void pad_cm_corner_kernel(ImgGeom g, const float2* __restrict__ xx,
                                     float2* __restrict__ pad, int64_t slabsz, int apply_sn,
                                     int dom_axis, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n0, n1;
    row_index<3>(r, g.N[0], g.N[1], inst, n0, n1);
    const int NL = g.N[2], B = g.B;
    const float s_lead = apply_sn ? lead_sn<3>(g.sn[0], g.sn[1], n0, n1) : 1.f;
    const float a_lead = (dom_axis == 0) ? (float)n0 - 0.5f * (float)g.N[0]
                         : (dom_axis == 1) ? (float)n1 - 0.5f * (float)g.N[1] : 0.f;
    const float2* src = xx + (size_t)r * NL * B;
    const size_t cell = ((size_t)n0 * g.K[1] + n1) * g.K[2];
    for (int e = threadIdx.x; e < NL * B; e += blockDim.x) {
        const int b = e / NL, k = e - b * NL;
        float2 v = __ldg(src + (size_t)k * B + b);
        if (apply_sn) {
            const float sc = s_lead * __ldg(g.sn[2] + k);
            v.x *= sc;
            v.y *= sc;
        }
        if (dom_axis >= 0) {   // x -i (n_a - N_a/2): the trajectory derivative
            const float a = (dom_axis == 2) ? (float)k - 0.5f * (float)NL : a_lead;
            v = make_float2(a * v.y, -a * v.x);
        }
        pad[((size_t)inst * B + b) * slabsz + cell + k] = v;
    }
  }
}

// Several coils, interleaved spectra: image row (n0[, n1]) of every coil
// into the zero-kept padded input (slab n0 B + b, only the Nd corner; the
// rest is never written), x sn, x -i (n_a - N_a/2) for the trajectory
// derivative.
template <int DIM>
__global__ void pad_il_kernel(ImgGeom g, const float2* __restrict__ xx, float2* __restrict__ pad,
                              int apply_sn, int dom_axis, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    constexpr int last = DIM - 1;
    const int NL = g.N[last], B = g.B;
    const float s_lead = apply_sn ? lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]) : 1.f;
    float a_lead = 0.f;
    if (dom_axis == 0) a_lead = (float)n[0] - 0.5f * (float)g.N[0];
    if (DIM == 3 && dom_axis == 1) a_lead = (float)n[1] - 0.5f * (float)g.N[1];
    const float2* src = xx + (size_t)r * NL * B;
    for (int e = threadIdx.x; e < NL * B; e += blockDim.x) {
        const int b = e / NL, k = e - b * NL;
        float2 v = __ldg(src + (size_t)k * B + b);
        if (apply_sn) {
            const float sc = s_lead * __ldg(g.sn[last] + k);
            v.x *= sc;
            v.y *= sc;
        }
        if (dom_axis >= 0) {
            const float a = (dom_axis == last) ? (float)k - 0.5f * (float)NL : a_lead;
            v = make_float2(a * v.y, -a * v.x);
        }
        pad[cm_at<DIM>(g, 0, b, n[0], n[1], k)] = v;
    }
  }
}

// Crop from coil-major spectra: one block per image row writes that row of
// every coil into the coil-fastest image (x 1/prod(Kd), x sn if apply_sn,
// / sn if divide_sn).
template <int DIM>
__global__ void crop_cm_rows_kernel(ImgGeom g, const float2* __restrict__ cm, float2* __restrict__ xx,
                                    int apply_sn, int divide_sn, float norm, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    const float s_lead = lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]);
    float2* dst = xx + (size_t)r * NL * B;
    for (int e = threadIdx.x; e < NL * B; e += blockDim.x) {
        const int b = e / NL, k = e - b * NL;
        float2 v = __ldg(cm + cm_at<DIM>(g, inst, b, n[0], n[1], k));
        float sc = norm;
        const float snv = s_lead * __ldg(g.sn[last] + k);
        if (apply_sn) sc *= snv;
        v.x *= sc;
        v.y *= sc;
        if (divide_sn) {
            v.x /= snv;
            v.y /= snv;
        }
        dst[(size_t)k * B + b] = v;
    }
  }
}

// SENSE coil expansion fused into x2xx + zero-pad (forward_one2many of the
// deprecated reference class, linalg/nufft_cpu.py:177-189): the single-coil
// image x (Nd) times each coil map (Nd, B) times sn, written into the
// B-coil grid row.
template <int DIM>
__global__ void pad_sense_rows_kernel(ImgGeom g, const float2* __restrict__ x,
                                      const float2* __restrict__ maps, float2* __restrict__ grid,
                                      int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.K[0], g.K[1], inst, n[0], n[1]);
    bool inside = true;
#pragma unroll
    for (int d = 0; d < DIM - 1; ++d) inside = inside && (n[d] < g.N[d]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    float2* dst = grid + (size_t)r * KL * B;
    if (!inside) {
        for (int e = threadIdx.x; e < KL * B; e += blockDim.x) dst[e] = make_float2(0.f, 0.f);
        continue;
    }
    float s_lead = 1.f;
    for (int d = 0; d < last; ++d) s_lead *= __ldg(g.sn[d] + n[d]);
    int64_t xrow = inst;
    for (int d = 0; d < last; ++d) xrow = xrow * g.N[d] + n[d];
    const float2* xs = x + (size_t)xrow * NL;
    const float2* ms = maps + (size_t)xrow * NL * B;      // single-instance plans only
    for (int e = threadIdx.x; e < KL * B; e += blockDim.x) {
        const int k = e / B;
        float2 v = make_float2(0.f, 0.f);
        if (k < NL) {
            const float2 a = __ldg(xs + k), m = __ldg(ms + e);
            const float sc = s_lead * __ldg(g.sn[last] + k);
            v = make_float2(sc * (a.x * m.x - a.y * m.y), sc * (a.x * m.y + a.y * m.x));
        }
        dst[e] = v;
    }
  }
}

// Coil combination fused into crop + xx2x (adjoint_many2one of the
// deprecated reference class, linalg/nufft_cpu.py:191-203):
// x[n] = mean_b conj(map[n,b]) * grid[n,b] * sn[n] / prod(Kd).
template <int DIM>
__global__ void crop_sense_rows_kernel(ImgGeom g, const float2* __restrict__ grid,
                                       const float2* __restrict__ maps, float2* __restrict__ x,
                                       float norm, int64_t rows) {
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    int64_t inst;
    int n[3] = {0, 0, 0};
    row_index<DIM>(r, g.N[0], g.N[1], inst, n[0], n[1]);
    constexpr int last = DIM - 1;
    const int KL = g.K[last], NL = g.N[last];
    const int B = g.B;
    const float s_lead = lead_sn<DIM>(g.sn[0], g.sn[1], n[0], n[1]);
    int64_t krow = inst;
#pragma unroll
    for (int d = 0; d < last; ++d) krow = krow * g.K[d] + n[d];
    const float2* src = grid + (size_t)krow * KL * B;
    const float2* ms = maps + (size_t)r * NL * B;         // single-instance plans only
    float2* dst = x + (size_t)r * NL;
    for (int k = threadIdx.x; k < NL; k += blockDim.x) {
        float ax = 0.f, ay = 0.f;
        for (int b = 0; b < B; ++b) {
            const float2 v = __ldg(src + (size_t)k * B + b), m = __ldg(ms + (size_t)k * B + b);
            ax = fmaf(m.x, v.x, fmaf(m.y, v.y, ax));      // conj(m) * v
            ay = fmaf(m.x, v.y, fmaf(-m.y, v.x, ay));
        }
        const float sc = norm * s_lead * __ldg(g.sn[last] + k) / (float)B;
        dst[k] = make_float2(ax * sc, ay * sc);
    }
  }
}

static int64_t rows_of(const ImgGeom& g, const int* ext, int ninst) {
    int64_t r = ninst;
    for (int d = 0; d < g.ndim - 1; ++d) r *= ext[d];
    return r;
}

static unsigned row_blocks(const nufft_plan_s* p, int64_t rows) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t)p->num_sms * 8));
}

static int row_threads(int len) {
    int t = 32;
    while (t < len && t < 256) t <<= 1;
    return t;
}

int launch_scale(const nufft_plan_s* p, const float2* in, float2* out, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const int64_t rows = rows_of(g, g.N, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.N[g.ndim - 1] * g.B);
    switch (p->ndim) {
        case 1: scale_rows_kernel<1><<<nb, nt, 0, s>>>(g, in, out, rows); break;
        case 2: scale_rows_kernel<2><<<nb, nt, 0, s>>>(g, in, out, rows); break;
        default: scale_rows_kernel<3><<<nb, nt, 0, s>>>(g, in, out, rows); break;
    }
    return check_launch("scale_rows_kernel");
}

int launch_pad(const nufft_plan_s* p, const float2* xx, float2* grid, bool apply_sn,
               int dom_axis, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const int64_t rows = rows_of(g, g.K, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.K[g.ndim - 1] * g.B);
    const int as = apply_sn ? 1 : 0;
    switch (p->ndim) {
        case 1: pad_rows_kernel<1><<<nb, nt, 0, s>>>(g, xx, grid, as, dom_axis, rows); break;
        case 2: pad_rows_kernel<2><<<nb, nt, 0, s>>>(g, xx, grid, as, dom_axis, rows); break;
        default: pad_rows_kernel<3><<<nb, nt, 0, s>>>(g, xx, grid, as, dom_axis, rows); break;
    }
    return check_launch("pad_rows_kernel");
}

static int coil_transpose(const nufft_plan_s* p, const float2* in, float2* out, bool to_major,
                          cudaStream_t s);

// Transforms of the coil-major spectra: per system the pruned slab + x-axis
// FFTs (3D plans with at most 16 systems), else one batched plan.
static int fft_cm_exec(nufft_plan_s* p, int direction, cudaStream_t s) {
    const int dir = (direction < 0) ? CUFFT_FORWARD : CUFFT_INVERSE;
    cufftComplex* cm = reinterpret_cast<cufftComplex*>(p->d_cm);
    if (p->cm_il && dir == CUFFT_INVERSE) {
        // columns, then only the first Nd[0] rows of every coil (the crop
        // reads nothing else)
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_cols, s));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_rows, s));
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_cols, cm, cm, dir));
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_rows, cm, cm, dir));
        return NUFFT_OK;
    }
    if (p->fft_cm_pruned) {
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_slab, s));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_x, s));
        const int S = p->ninst * p->B;
        for (int i = 0; i < S; ++i) {
            cufftComplex* gi = cm + (size_t)i * p->prodK;
            if (dir == CUFFT_FORWARD) {
                NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, gi, gi, dir));
                NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, gi, gi, dir));
            } else {
                NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, gi, gi, dir));
                NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, gi, gi, dir));
            }
        }
        return NUFFT_OK;
    }
    NUFFT_CUFFT_TRY(cufftSetStream(p->fft, s));
    NUFFT_CUFFT_TRY(cufftExecC2C(p->fft, cm, cm, dir));
    return NUFFT_OK;
}

// Several coils: the coil-major spectra in p->d_cm -> image xx (coil-fastest):
// inverse FFTs in place, then the crop straight from the coil-major spectra
// (x sn when apply_sn, / sn when divide_sn, / prod(Kd)).
int cm_to_image(nufft_plan_s* p, float2* xx, bool apply_sn, bool divide_sn, cudaStream_t s) {
    NUFFT_TRY(fft_cm_exec(p, +1, s));
    ImgGeom g = img_geom(p);
    const float norm = (float)(1.0 / (double)p->prodK);
    const int64_t rows = rows_of(g, g.N, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.N[g.ndim - 1] * g.B);
    const int as = apply_sn ? 1 : 0, ds = divide_sn ? 1 : 0;
    switch (p->ndim) {
        case 1: crop_cm_rows_kernel<1><<<nb, nt, 0, s>>>(g, p->d_cm, xx, as, ds, norm, rows); break;
        case 2: crop_cm_rows_kernel<2><<<nb, nt, 0, s>>>(g, p->d_cm, xx, as, ds, norm, rows); break;
        default: crop_cm_rows_kernel<3><<<nb, nt, 0, s>>>(g, p->d_cm, xx, as, ds, norm, rows); break;
    }
    return check_launch("crop_cm_rows_kernel");
}

// Several coils: spectrum k (coil-fastest) -> image xx (coil-fastest):
// transpose to coil-major, then cm_to_image.  k is read only.
int image_from_spectrum_coils(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn,
                              bool divide_sn, cudaStream_t s) {
    if (p->cfft) return cfft_inverse(p, k, xx, apply_sn, divide_sn, s);
    NUFFT_TRY(coil_transpose(p, k, p->d_cm, true, s));
    return cm_to_image(p, xx, apply_sn, divide_sn, s);
}

int cm_to_grid(const nufft_plan_s* p, float2* k, cudaStream_t s) {
    return coil_transpose(p, p->d_cm, k, false, s);
}

// Several coils: image xx (coil-fastest) -> coil-major spectra in p->d_cm:
// every coil's grid padded straight into the coil-major buffer (x sn when
// apply_sn), then the forward FFTs in place.
int image_to_cm(nufft_plan_s* p, const float2* xx, bool apply_sn, cudaStream_t s, int dom_axis) {
    ImgGeom g = img_geom(p);
    if (p->cm_il) {
        // interleaved: the image corner into the zero-kept padded slabs,
        // their (inner-axes) FFTs into the zero-kept slab buffer, its
        // first-axis FFTs into the coil-major spectra
        // (the padded input holds the first Nd[0] slabs of every coil, laid
        // out like the spectra's first Nd[0] B slabs)
        const int64_t rows = rows_of(g, g.N, 1);
        const unsigned nb = row_blocks(p, rows);
        const int nt = row_threads(g.N[g.ndim - 1] * g.B);
        const int as = apply_sn ? 1 : 0;
        if (p->ndim == 2)
            pad_il_kernel<2><<<nb, nt, 0, s>>>(g, xx, p->d_il_pad, as, dom_axis, rows);
        else
            pad_il_kernel<3><<<nb, nt, 0, s>>>(g, xx, p->d_il_pad, as, dom_axis, rows);
        NUFFT_TRY(check_launch("pad_il_kernel"));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_rows, s));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_cols, s));
        cufftComplex* pad = reinterpret_cast<cufftComplex*>(p->d_il_pad);
        cufftComplex* z = reinterpret_cast<cufftComplex*>(p->d_il_z);
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_rows, pad, z, CUFFT_FORWARD));
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_cols, z, reinterpret_cast<cufftComplex*>(p->d_cm),
                                     CUFFT_FORWARD));
        return NUFFT_OK;
    }
    if (p->fft_cm_pruned && p->d_cmpad) {
        // 3D, a few systems: write only the Nd corners into the zero-kept
        // padded inputs; per system the (y, z) FFTs of its N0 slabs run out of
        // place into the zero-kept slab buffer and the x-axis FFTs from there
        // into the system's coil-major spectrum
        const int64_t rows = rows_of(g, g.N, p->ninst);
        const int64_t slabsz = (int64_t)p->Nd[0] * (p->prodK / p->Kd[0]);
        pad_cm_corner_kernel<<<row_blocks(p, rows), row_threads(g.N[2] * g.B), 0, s>>>(
            g, xx, p->d_cmpad, slabsz, apply_sn ? 1 : 0, dom_axis, rows);
        NUFFT_TRY(check_launch("pad_cm_corner_kernel"));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_slab, s));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_x, s));
        cufftComplex* slab = reinterpret_cast<cufftComplex*>(p->d_cmslab);
        for (int i = 0; i < p->ninst * p->B; ++i) {
            cufftComplex* in = reinterpret_cast<cufftComplex*>(p->d_cmpad) + (size_t)i * slabsz;
            cufftComplex* out = reinterpret_cast<cufftComplex*>(p->d_cm) + (size_t)i * p->prodK;
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, in, slab, CUFFT_FORWARD));
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, slab, out, CUFFT_FORWARD));
        }
        return NUFFT_OK;
    }
    const int64_t rows = rows_of(g, g.K, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.K[g.ndim - 1] * g.B);
    const int as = apply_sn ? 1 : 0;
    switch (p->ndim) {
        case 1: pad_cm_rows_kernel<1><<<nb, nt, 0, s>>>(g, xx, p->d_cm, as, dom_axis, rows); break;
        case 2: pad_cm_rows_kernel<2><<<nb, nt, 0, s>>>(g, xx, p->d_cm, as, dom_axis, rows); break;
        default: pad_cm_rows_kernel<3><<<nb, nt, 0, s>>>(g, xx, p->d_cm, as, dom_axis, rows); break;
    }
    NUFFT_TRY(check_launch("pad_cm_rows_kernel"));
    return fft_cm_exec(p, -1, s);
}

// Image (Nd, caller's layout) -> oversampled spectrum k: zero-pad (x sn when
// apply_sn) and forward FFT.  For one coil and one instance the pad only
// writes the Nd corner of the plan's padded input buffer (its zeros are
// never overwritten), the (y[,z]) FFTs run out of place on its first Nd[0]
// slabs into the slab buffer (whose other slabs stay zero), and the x-axis
// FFTs write k: the 134 MB zero fill of a 256^3 grid is not rewritten on
// every call.
int forward_from_image(nufft_plan_s* p, const float2* xx, bool apply_sn, float2* k,
                       cudaStream_t s, int dom_axis) {
    if (p->cfft) return cfft_forward(p, xx, apply_sn, dom_axis, k, s);
    if (p->B > 1) {
        // coil-major: pad every coil's grid, transform there, transpose to k
        NUFFT_TRY(image_to_cm(p, xx, apply_sn, s, dom_axis));
        return coil_transpose(p, p->d_cm, k, false, s);
    }
    if (dom_axis >= 0) {
        NUFFT_TRY(launch_pad(p, xx, k, apply_sn, dom_axis, s));
        return fft_exec(p, k, -1, s);
    }
    if (p->pfft) return pfft_forward(p, xx, apply_sn, k, s);
    if (!(p->fft_pruned && p->d_padin)) {
        NUFFT_TRY(launch_pad(p, xx, k, apply_sn, -1, s));
        return fft_exec(p, k, -1, s);
    }
    ImgGeom g = img_geom(p);
    const int64_t rows = rows_of(g, g.N, 1);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.N[g.ndim - 1]);
    const int as = apply_sn ? 1 : 0;
    if (p->ndim == 2)
        corner_rows_kernel<2><<<nb, nt, 0, s>>>(g, xx, p->d_padin, as, rows);
    else
        corner_rows_kernel<3><<<nb, nt, 0, s>>>(g, xx, p->d_padin, as, rows);
    NUFFT_TRY(check_launch("corner_rows_kernel"));
    cufftComplex* a = reinterpret_cast<cufftComplex*>(p->d_padin);
    cufftComplex* b = reinterpret_cast<cufftComplex*>(p->d_slabout);
    cufftComplex* kc = reinterpret_cast<cufftComplex*>(k);
    NUFFT_CUFFT_TRY(cufftSetStream(p->fft_slab, s));
    NUFFT_CUFFT_TRY(cufftSetStream(p->fft_x, s));
    NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, a, b, CUFFT_FORWARD));
    NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, b, kc, CUFFT_FORWARD));
    return NUFFT_OK;
}

// The own coil-batched passes (2D, several coils), the own pruned passes
// (one coil), else the inverse cuFFT in place on k followed by the crop.
int image_from_spectrum(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn,
                        bool divide_sn, cudaStream_t s) {
    if (p->cfft) return cfft_inverse(p, k, xx, apply_sn, divide_sn, s);
    if (p->pfft) return pfft_inverse(p, k, xx, apply_sn, divide_sn, s);
    float2* kk = const_cast<float2*>(k);
    NUFFT_TRY(fft_exec(p, kk, +1, s));
    return launch_crop(p, kk, xx, apply_sn, divide_sn, s);
}

int launch_crop(const nufft_plan_s* p, const float2* grid, float2* xx, bool apply_sn,
                bool divide_sn, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const float norm = (float)(1.0 / (double)p->prodK);
    const int64_t rows = rows_of(g, g.N, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.N[g.ndim - 1] * g.B);
    const int as = apply_sn ? 1 : 0, ds = divide_sn ? 1 : 0;
    switch (p->ndim) {
        case 1: crop_rows_kernel<1><<<nb, nt, 0, s>>>(g, grid, xx, as, ds, norm, rows); break;
        case 2: crop_rows_kernel<2><<<nb, nt, 0, s>>>(g, grid, xx, as, ds, norm, rows); break;
        default: crop_rows_kernel<3><<<nb, nt, 0, s>>>(g, grid, xx, as, ds, norm, rows); break;
    }
    return check_launch("crop_rows_kernel");
}

// Coil-fastest grid (cells, B) <-> coil-major (B, cells), per instance
// (blockIdx.y), through a shared tile of R cells x B coils (R B ~ 1024):
// both the global reads and the global writes run along contiguous memory.
__global__ void to_coil_major_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                     int64_t cells, int B, int R) {
    extern __shared__ float2 t[];   // B x (R + 1)
    const int64_t c0 = (int64_t)blockIdx.x * R;
    const size_t off = (size_t)blockIdx.y * cells * B;
    const int n = R * B;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int r = e / B, b = e - r * B;
        if (c0 + r < cells) t[b * (R + 1) + r] = in[off + (size_t)(c0 + r) * B + b];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int b = e / R, r = e - b * R;
        if (c0 + r < cells) out[off + (size_t)b * cells + c0 + r] = t[b * (R + 1) + r];
    }
}

__global__ void to_coil_fast_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                    int64_t cells, int B, int R) {
    extern __shared__ float2 t[];   // B x (R + 1)
    const int64_t c0 = (int64_t)blockIdx.x * R;
    const size_t off = (size_t)blockIdx.y * cells * B;
    const int n = R * B;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int b = e / R, r = e - b * R;
        if (c0 + r < cells) t[b * (R + 1) + r] = in[off + (size_t)b * cells + c0 + r];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int r = e / B, b = e - r * B;
        if (c0 + r < cells) out[off + (size_t)(c0 + r) * B + b] = t[b * (R + 1) + r];
    }
}

static int coil_transpose(const nufft_plan_s* p, const float2* in, float2* out, bool to_major,
                          cudaStream_t s) {
    const int B = p->B;
    const int R = std::max(1, 2048 / B);   // 2048-element tiles (1024: 8-coil kooshball forward
                                           // 10.91 ms, 2048: 10.77, 4096: 10.96)
    // interleaved spectra: every first-axis slab on its own (prod(Kd) / K0
    // cells x B coils)
    const int64_t cells = p->cm_il ? p->prodK / p->Kd[0] : p->prodK;
    const dim3 grid((unsigned)((cells + R - 1) / R), (unsigned)(p->cm_il ? p->Kd[0] : p->ninst));
    const size_t smem = sizeof(float2) * (size_t)B * (R + 1);
    if (to_major)
        to_coil_major_kernel<<<grid, 256, smem, s>>>(in, out, cells, B, R);
    else
        to_coil_fast_kernel<<<grid, 256, smem, s>>>(in, out, cells, B, R);
    return check_launch("coil transpose");
}

// cuFFT plans.  The general plan transforms all axes of every coil and
// instance.  For one coil and one instance the zero padding is exploited:
// the forward transform runs the (y[,z]) FFTs only on the first N0 slabs
// (the others are zero) and then the x-axis FFTs; the inverse runs the x-axis
// FFTs and then the (y[,z]) FFTs only on the N0 slabs the crop keeps.  All
// plans share one work area.
static int make_plan(cufftHandle* h, int rank, int* n, int stride, int dist, int batch,
                     size_t* work) {
    NUFFT_CUFFT_TRY(cufftCreate(h));
    NUFFT_CUFFT_TRY(cufftSetAutoAllocation(*h, 0));
    size_t ws = 0;
    NUFFT_CUFFT_TRY(cufftMakePlanMany(*h, rank, n, n, stride, dist, n, stride, dist, CUFFT_C2C,
                                      batch, &ws));
    *work = std::max(*work, ws);
    return NUFFT_OK;
}

// A plan over embedded arrays: logical sizes n, storage inembed (= onembed).
static int make_plan_embed(cufftHandle* h, int rank, int* n, int* embed, int stride, int dist,
                           int batch, size_t* work) {
    NUFFT_CUFFT_TRY(cufftCreate(h));
    NUFFT_CUFFT_TRY(cufftSetAutoAllocation(*h, 0));
    size_t ws = 0;
    NUFFT_CUFFT_TRY(cufftMakePlanMany(*h, rank, n, embed, stride, dist, embed, stride, dist,
                                      CUFFT_C2C, batch, &ws));
    *work = std::max(*work, ws);
    return NUFFT_OK;
}

int launch_pad_sense(const nufft_plan_s* p, const float2* x, float2* grid, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const int64_t rows = rows_of(g, g.K, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.K[g.ndim - 1] * g.B);
    switch (p->ndim) {
        case 1: pad_sense_rows_kernel<1><<<nb, nt, 0, s>>>(g, x, p->d_maps, grid, rows); break;
        case 2: pad_sense_rows_kernel<2><<<nb, nt, 0, s>>>(g, x, p->d_maps, grid, rows); break;
        default: pad_sense_rows_kernel<3><<<nb, nt, 0, s>>>(g, x, p->d_maps, grid, rows); break;
    }
    return check_launch("pad_sense_rows_kernel");
}

int launch_crop_sense(const nufft_plan_s* p, const float2* grid, float2* x, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const float norm = (float)(1.0 / (double)p->prodK);
    const int64_t rows = rows_of(g, g.N, p->ninst);
    const unsigned nb = row_blocks(p, rows);
    const int nt = row_threads(g.N[g.ndim - 1]);
    switch (p->ndim) {
        case 1: crop_sense_rows_kernel<1><<<nb, nt, 0, s>>>(g, grid, p->d_maps, x, norm, rows); break;
        case 2: crop_sense_rows_kernel<2><<<nb, nt, 0, s>>>(g, grid, p->d_maps, x, norm, rows); break;
        default: crop_sense_rows_kernel<3><<<nb, nt, 0, s>>>(g, grid, p->d_maps, x, norm, rows); break;
    }
    return check_launch("crop_sense_rows_kernel");
}

int fft_init(nufft_plan_s* p) {
    int n[3] = {p->Kd[0], p->Kd[1], p->Kd[2]};
    const int B = p->B;
    size_t work = 0;
    // one contiguous batched plan over every coil-major grid (B > 1 transforms
    // go through a coil-major copy: cuFFT's coil-strided transforms ran at
    // under 1 TB/s); 2D plans of several coils and one instance keep the
    // copy row-interleaved (nufft_plan_s::cm_il)
    // (3D: only up to 1 GiB of spectra -- 8 coils at 192^3: pair 3.95 -> 3.74
    // ms; at 384^3, 3.6 GB, the per-system pruned plans below were 1.5%
    // faster: 31.1 against 31.5 ms)
    p->cfft = cfft_eligible(p);
    p->cm_il = (!p->cfft && B > 1 && p->ninst == 1 &&
                (p->ndim == 2 ||
                 (p->ndim == 3 && sizeof(float2) * (size_t)B * p->prodK <= ((size_t)1 << 30))));
    if (p->cm_il) {
        const int slab = (int)(p->prodK / p->Kd[0]);   // cells of a first-axis slab
        int embed[3] = {p->Kd[0], B * p->Kd[1], p->ndim == 3 ? p->Kd[2] : 1};
        NUFFT_TRY(make_plan_embed(&p->fft, p->ndim, n, embed, 1, slab, B, &work));
        NUFFT_TRY(make_plan(&p->fft_rows, p->ndim - 1, n + 1, 1, slab, p->Nd[0] * B, &work));
        int nc[1] = {p->Kd[0]};
        NUFFT_TRY(make_plan_embed(&p->fft_cols, 1, nc, nc, B * slab, 1, B * slab, &work));
    } else {
        NUFFT_TRY(make_plan(&p->fft, p->ndim, n, 1, (int)p->prodK, p->ninst * B, &work));
    }
    if (B > 1) {
        const size_t ncm = (size_t)p->ninst * B * p->prodK;
        if (B > 1024 || ncm > ((size_t)1 << 40)) {
            set_error("nufft_plan_create: unsupported batch for the coil-major FFT");
            return NUFFT_EUNSUPPORTED;
        }
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_cm, sizeof(float2) * ncm));
        p->dev_bytes += sizeof(float2) * ncm;
    }
    p->fft_ok = true;
    if (B == 1 && p->ninst == 1 && p->ndim >= 2 && p->Nd[0] < p->Kd[0]) {
        const int slab = (int)(p->prodK / p->Kd[0]);
        NUFFT_TRY(make_plan(&p->fft_slab, p->ndim - 1, n + 1, 1, slab, p->Nd[0], &work));
        NUFFT_TRY(make_plan(&p->fft_x, 1, n, slab, 1, slab, &work));
        p->fft_pruned = true;
    } else if (B > 1 && !p->cm_il && !p->cfft && p->ndim == 3 && p->Nd[0] < p->Kd[0] &&
               p->ninst * B <= 16) {
        // coil-major spectra of a few 3D systems: the same pruned pair of
        // plans, run once per system
        const int slab = (int)(p->prodK / p->Kd[0]);
        NUFFT_TRY(make_plan(&p->fft_slab, p->ndim - 1, n + 1, 1, slab, p->Nd[0], &work));
        NUFFT_TRY(make_plan(&p->fft_x, 1, n, slab, 1, slab, &work));
        p->fft_cm_pruned = true;
    }
    if (work > 0) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_fftwork, work));
        p->dev_bytes += work;
    }
    if (p->cm_il) {
        // zero-kept padded slabs (Nd[0] B of them) and slab-FFT output (K0 B)
        const size_t npad = (size_t)p->Nd[0] * B * (p->prodK / p->Kd[0]);
        const size_t nz = (size_t)p->prodK * B;
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_il_pad, sizeof(float2) * npad));
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_il_z, sizeof(float2) * nz));
        NUFFT_CUDA_TRY(cudaMemset(p->d_il_pad, 0, sizeof(float2) * npad));
        NUFFT_CUDA_TRY(cudaMemset(p->d_il_z, 0, sizeof(float2) * nz));
        p->dev_bytes += sizeof(float2) * (npad + nz);
    }
    if (p->fft_cm_pruned) {
        // per system a padded input (first Nd[0] slabs), one shared slab-FFT
        // output; both zero once, only their Nd corner / first Nd[0] slabs
        // are ever written
        const size_t nin = (size_t)p->ninst * B * p->Nd[0] * (p->prodK / p->Kd[0]);
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_cmpad, sizeof(float2) * nin));
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_cmslab, sizeof(float2) * p->prodK));
        NUFFT_CUDA_TRY(cudaMemset(p->d_cmpad, 0, sizeof(float2) * nin));
        NUFFT_CUDA_TRY(cudaMemset(p->d_cmslab, 0, sizeof(float2) * p->prodK));
        p->dev_bytes += sizeof(float2) * (nin + p->prodK);
    }
    if (p->fft_pruned) {
        // padded input (first Nd[0] slabs) and slab-FFT output, zero once
        const size_t nin = (size_t)p->Nd[0] * (p->prodK / p->Kd[0]);
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_padin, sizeof(float2) * nin));
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_slabout, sizeof(float2) * p->prodK));
        NUFFT_CUDA_TRY(cudaMemset(p->d_padin, 0, sizeof(float2) * nin));
        NUFFT_CUDA_TRY(cudaMemset(p->d_slabout, 0, sizeof(float2) * p->prodK));
        p->dev_bytes += sizeof(float2) * (nin + p->prodK);
    }
    NUFFT_CUFFT_TRY(cufftSetWorkArea(p->fft, p->d_fftwork));
    if (p->fft_pruned || p->fft_cm_pruned) {
        NUFFT_CUFFT_TRY(cufftSetWorkArea(p->fft_slab, p->d_fftwork));
        NUFFT_CUFFT_TRY(cufftSetWorkArea(p->fft_x, p->d_fftwork));
    }
    if (p->cm_il) {
        NUFFT_CUFFT_TRY(cufftSetWorkArea(p->fft_rows, p->d_fftwork));
        NUFFT_CUFFT_TRY(cufftSetWorkArea(p->fft_cols, p->d_fftwork));
    }
    NUFFT_TRY(cfft_init(p));
    // own pruned passes where the grid allows (they use d_padin / d_slabout
    // as their intermediate arrays)
    return pfft_init(p);
}

void fft_destroy(nufft_plan_s* p) {
    if (p->fft_ok) cufftDestroy(p->fft);
    if (p->fft_pruned || p->fft_cm_pruned) {
        cufftDestroy(p->fft_slab);
        cufftDestroy(p->fft_x);
    }
    if (p->cm_il) {
        cufftDestroy(p->fft_rows);
        cufftDestroy(p->fft_cols);
    }
    p->fft_ok = p->fft_pruned = p->fft_cm_pruned = p->cm_il = false;
    cudaFree(p->d_il_pad);
    cudaFree(p->d_il_z);
    p->d_il_pad = p->d_il_z = nullptr;
    pfft_free(p);
    cfft_free(p);
    cudaFree(p->d_fftwork);
    p->d_fftwork = nullptr;
    cudaFree(p->d_padin);
    cudaFree(p->d_slabout);
    cudaFree(p->d_cm);
    cudaFree(p->d_cmpad);
    cudaFree(p->d_cmslab);
    p->d_padin = p->d_slabout = p->d_cm = p->d_cmpad = p->d_cmslab = nullptr;
}

// direction < 0: forward (numpy fftn sign); > 0: inverse, unnormalised.
// After an inverse transform of a single-coil plan only the first Nd[0]
// slabs hold the transform (the crop reads nothing else).
int fft_exec(nufft_plan_s* p, float2* grid, int direction, cudaStream_t s) {
    const int dir = (direction < 0) ? CUFFT_FORWARD : CUFFT_INVERSE;
    cufftComplex* gc = reinterpret_cast<cufftComplex*>(grid);
    if (p->fft_pruned) {
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_slab, s));
        NUFFT_CUFFT_TRY(cufftSetStream(p->fft_x, s));
        if (dir == CUFFT_FORWARD) {
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, gc, gc, dir));
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, gc, gc, dir));
        } else {
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_x, gc, gc, dir));
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft_slab, gc, gc, dir));
        }
        return NUFFT_OK;
    }
    NUFFT_CUFFT_TRY(cufftSetStream(p->fft, s));
    if (p->B == 1) {
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft, gc, gc, dir));
        return NUFFT_OK;
    }
    cufftComplex* cm = reinterpret_cast<cufftComplex*>(p->d_cm);
    NUFFT_TRY(coil_transpose(p, grid, p->d_cm, true, s));
    NUFFT_CUFFT_TRY(cufftExecC2C(p->fft, cm, cm, dir));
    return coil_transpose(p, p->d_cm, grid, false, s);
}

}  // namespace nufft

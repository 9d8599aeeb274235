// Coil-batched FFT passes on coil-fastest layouts: the image <-> spectrum
// transforms of 2D and 3D plans of several coils (a multiple of 8) and one
// instance, with every Kd in {128, 160, 192, 256, 320, 384, 512, 640}.
//
// The reference's batch layout keeps the coil index fastest in the image,
// the spectrum and the samples (linalg/nufft_hsa.py:203-228).  These passes
// transform that layout in place of the coil-major copy, transposes and
// cuFFT calls: one pass per axis, each a set of L-point transforms along a
// strided axis whose batch (coils, or coils x cells) is contiguous.  A block
// takes 8 contiguous batch elements (64 bytes per row) and runs their 8
// transforms together: a mixed-radix Stockham FFT in three radix stages
// (640 = 10 x 8 x 8, 512 = 8 x 8 x 8, 384 = 6 x 8 x 8, 320 = 5 x 8 x 8,
// 256 = 4 x 8 x 8, 192 = 6 x 4 x 8, 160 = 5 x 4 x 8, 128 = 2 x 8 x 8),
// the first reading global memory, the last writing it, shared memory in
// between, twiddles from a plan-time table.  Zero padding and cropping are
// pruned (the first stage reads only the `lin` nonzero inputs, the last
// writes only the `lout` kept outputs), and the image side is fused:
//
//   forward  image x[n0][n1][b] --(rows, x sn, -i(n_a - N_a/2) for the
//            trajectory derivative)--> mid[n0][k1][b] --(columns)--> k[k0][k1][b]
//   inverse  k[k0][k1][b] --(columns, k0 -> n0 < N0)--> mid[n0][k1][b]
//            --(rows, k1 -> n1 < N1, x 1/prod(Kd), x sn or / sn)--> x[n0][n1][b]
//
// and in 3D the same with three passes (z on the image's rows, then y, then
// x), each reading only the slabs the previous one left nonzero.  The
// intermediate arrays live in the plan's coil-major buffer, which these
// plans do not otherwise use.
//
// (the reference's xx2k / k2xx: zero-pad into the top-left corner and
// numpy.fft.fftn / ifftn, nufft/_nufft_class_methods_cpu.py:232-249, 316-329).
#include "nufft_internal.cuh"
#include "cfft_dft.cuh"

#include <cmath>
#include <vector>

namespace nufft {
namespace {

using cdft::kCW;
using cdft::Plan3;

// Element offsets fit 32 bits (the plans these passes serve hold fewer than
// 2^31 grid elements), and the batch is a multiple of kCW.
struct CfftArgs {
    const float2* in;
    float2* out;
    int in_so, in_sl;        // input strides (elements) of the outer and transform indices
    int out_so, out_sl;      // output strides
    int inner;               // batch elements per (outer, index)
    int nchunk;              // blocks per outer index: inner / kCW
    int lin, lout;           // inputs read (the rest are zero), outputs written
    const float2* tw;        // exp(-2 pi i m / L), m < L
    // image side (the pass along the last axis): MODE 1 scales the input,
    // MODE 2 the output.  The outer index o is (oa, ob) = (o / nob, o % nob):
    // n0 in 2D (nob = 1), (n0, n1) in 3D; l is the last axis's index.
    const float* sn_a;
    const float* sn_b;       // null in 2D
    const float* sn_l;
    int nob;
    int apply_sn, divide_sn;
    int dom;                 // -1, or the index the trajectory derivative multiplies by:
                             // 0 oa, 1 ob, 2 l
    float dom_half;          // N_a / 2 of that axis
    float norm;
    // MODE 3 (the first inverse pass of a deterministic adjoint): `in` holds
    // the 64-bit fixed-point sums (re, im per element) that dscal[1] scales,
    // rounded here as the separate rounding kernel would
    const double* dscal;
};

template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2* tw, int m) {
    const float2 v = tw[m];
    return INV ? make_float2(v.x, -v.y) : v;
}

__device__ __forceinline__ float sn_at(const CfftArgs& a, int o, int l) {
    const int oa = o / a.nob, ob = o - oa * a.nob;
    float v = __ldg(a.sn_a + oa) * __ldg(a.sn_l + l);
    if (a.sn_b) v *= __ldg(a.sn_b + ob);
    return v;
}

template <int MODE>
__device__ __forceinline__ float2 pre_op(const CfftArgs& a, int o, int l, float2 v) {
    if constexpr (MODE == 1) {
        if (a.apply_sn) {
            const float sc = sn_at(a, o, l);
            v.x *= sc;
            v.y *= sc;
        }
        if (a.dom >= 0) {   // x -i (n_a - N_a / 2)
            const int oa = o / a.nob;
            const int n = (a.dom == 0) ? oa : (a.dom == 1) ? o - oa * a.nob : l;
            const float t = (float)n - a.dom_half;
            v = make_float2(t * v.y, -t * v.x);
        }
    }
    return v;
}

template <int MODE>
__device__ __forceinline__ float2 post_op(const CfftArgs& a, int o, int l, float2 v) {
    if constexpr (MODE == 2) {
        const float snv = sn_at(a, o, l);
        float sc = a.norm;
        if (a.apply_sn) sc *= snv;
        v.x *= sc;
        v.y *= sc;
        if (a.divide_sn) {
            v.x /= snv;
            v.y /= snv;
        }
    }
    return v;
}

// smem -> smem stage
template <typename P, typename S, int R, bool INV>
__device__ __forceinline__ void mid_stage(float2* buf, const float2* tw, int j, int w) {
    float2 v[R];
    const bool act = j < S::NB;
    if (act) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[r] = buf[P::row(S::in_index(j, r)) * kCW + w];
            if (r > 0) v[r] = cdft::mul(v[r], twiddle<INV>(tw, S::tw_index(j, r)));
        }
        cdft::dft<R, INV>(v);
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int r = 0; r < R; ++r) buf[P::row(S::out_index(j, r)) * kCW + w] = v[r];
    }
    __syncthreads();
}

// One pass: block = (outer index o, batch chunk); thread = (butterfly j,
// transform w).
template <int L, int R0, int R1, int R2, bool INV, int MODE>
__global__ void __launch_bounds__(Plan3<L, R0, R1, R2>::THREADS)
    cfft_pass_kernel(CfftArgs a) {
    using P = Plan3<L, R0, R1, R2>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);   // ROWS x kCW
    float2* tw = buf + P::ROWS * kCW;                     // L
    for (int m = threadIdx.x; m < L; m += blockDim.x) tw[m] = __ldg(a.tw + m);
    const int w = threadIdx.x % kCW, j = threadIdx.x / kCW;
    const int o = blockIdx.x / a.nchunk, ch = blockIdx.x - o * a.nchunk;
    const int e = ch * kCW + w;   // batch element
    const float2* __restrict__ in = a.in + (o * a.in_so + e);
    float2* __restrict__ out = a.out + (o * a.out_so + e);
    // MODE 3: (re, im) fixed-point pairs, 16 bytes per element
    const ulonglong2* __restrict__ fin =
        reinterpret_cast<const ulonglong2*>(a.in) + (o * a.in_so + e);
    float finv = 1.f;
    if constexpr (MODE == 3) finv = (float)(1.0 / __ldg(a.dscal + 1));

    {   // stage 0: global -> shared (inputs past lin are zero); the barrier
        // after it also publishes the twiddle table
        using S = typename P::S0;
        if (j < S::NB) {
            float2 v[R0];
#pragma unroll
            for (int r = 0; r < R0; ++r) {
                const int l = S::in_index(j, r);
                if constexpr (MODE == 3) {
                    if (l < a.lin) {
                        const ulonglong2 q = __ldg(fin + l * a.in_sl);
                        v[r] = make_float2(__ll2float_rn((long long)q.x) * finv,
                                           __ll2float_rn((long long)q.y) * finv);
                    } else {
                        v[r] = make_float2(0.f, 0.f);
                    }
                } else {
                    v[r] = (l < a.lin) ? pre_op<MODE>(a, o, l, __ldg(in + l * a.in_sl))
                                       : make_float2(0.f, 0.f);
                }
            }
            cdft::dft<R0, INV>(v);
#pragma unroll
            for (int r = 0; r < R0; ++r) buf[P::row(S::out_index(j, r)) * kCW + w] = v[r];
        }
        __syncthreads();
    }
    mid_stage<P, typename P::S1, R1, INV>(buf, tw, j, w);
    {   // last stage: shared -> global (outputs past lout are dropped)
        using S = typename P::S2;
        if (j < S::NB) {
            float2 v[R2];
#pragma unroll
            for (int r = 0; r < R2; ++r) {
                v[r] = buf[P::row(S::in_index(j, r)) * kCW + w];
                if (r > 0) v[r] = cdft::mul(v[r], twiddle<INV>(tw, S::tw_index(j, r)));
            }
            cdft::dft<R2, INV>(v);
#pragma unroll
            for (int r = 0; r < R2; ++r) {
                const int l = S::out_index(j, r);
                if (l < a.lout) out[l * a.out_sl] = post_op<MODE>(a, o, l, v[r]);
            }
        }
    }
}

template <int L, int R0, int R1, int R2, bool INV, int MODE>
int run_pass(const CfftArgs& a, int64_t outer, cudaStream_t s) {
    using P = Plan3<L, R0, R1, R2>;
    auto kern = cfft_pass_kernel<L, R0, R1, R2, INV, MODE>;
    NUFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)P::SMEM));
    const int64_t blocks = outer * a.nchunk;
    if (a.inner % kCW != 0 || blocks >= ((int64_t)1 << 31)) {
        set_error("cfft: batch not a multiple of 8 or too many blocks");
        return NUFFT_EUNSUPPORTED;
    }
    if (blocks > 0) kern<<<(unsigned)blocks, P::THREADS, P::SMEM, s>>>(a);
    return check_launch("cfft_pass_kernel");
}

template <bool INV, int MODE>
int run_len(int L, const CfftArgs& a, int64_t outer, cudaStream_t s) {
    switch (L) {
        case 640: return run_pass<640, 10, 8, 8, INV, MODE>(a, outer, s);
        case 512: return run_pass<512, 8, 8, 8, INV, MODE>(a, outer, s);
        case 384: return run_pass<384, 6, 8, 8, INV, MODE>(a, outer, s);
        case 320: return run_pass<320, 5, 8, 8, INV, MODE>(a, outer, s);
        case 256: return run_pass<256, 4, 8, 8, INV, MODE>(a, outer, s);
        case 192: return run_pass<192, 6, 4, 8, INV, MODE>(a, outer, s);
        case 160: return run_pass<160, 5, 4, 8, INV, MODE>(a, outer, s);
        case 128: return run_pass<128, 2, 8, 8, INV, MODE>(a, outer, s);
        default:
            set_error("cfft: unsupported transform length");
            return NUFFT_EUNSUPPORTED;
    }
}

bool length_ok(int L) {
    return L == 128 || L == 160 || L == 192 || L == 256 || L == 320 || L == 384 || L == 512 ||
           L == 640;
}

// the twiddle table of axis d
const float2* axis_tw(const nufft_plan_s* p, int d) {
    const float2* t = p->d_cfft_tw;
    for (int e = 0; e < d; ++e) t += p->Kd[e];
    return t;
}

// One pass along axis d of the coil-fastest array [outer][L][inner]:
// in[o][l][e] (strides in_so, in_sl) -> out[o][l][e].  The pass along the
// last axis carries the image side (sn, the trajectory derivative, the
// normalisation).
CfftArgs pass_args(const nufft_plan_s* p, const float2* in, float2* out, int d, int64_t in_so,
                   int64_t out_so, int64_t inner, int lin, int lout) {
    CfftArgs a{};
    a.in = in;
    a.out = out;
    a.in_so = (int)in_so;
    a.out_so = (int)out_so;
    a.in_sl = a.out_sl = (int)inner;
    a.inner = (int)inner;
    a.nchunk = (int)(inner / kCW);
    a.lin = lin;
    a.lout = lout;
    a.tw = axis_tw(p, d);
    a.sn_a = p->d_snd;
    a.sn_b = (p->ndim == 3) ? p->d_snd + p->Nd[0] : nullptr;
    a.sn_l = p->d_snd + (p->ndim == 3 ? p->Nd[0] + p->Nd[1] : p->Nd[0]);
    a.nob = (p->ndim == 3) ? p->Nd[1] : 1;
    a.dom = -1;
    a.norm = 1.f;
    return a;
}

}  // namespace

bool cfft_eligible(const nufft_plan_s* p) {
    if (p->flags & NUFFT_FLAG_CUFFT) return false;
    if ((p->ndim != 2 && p->ndim != 3) || p->ninst != 1 || p->B < 8 || p->B % kCW != 0)
        return false;
    for (int d = 0; d < p->ndim; ++d)
        if (!length_ok(p->Kd[d]) || p->Nd[d] > p->Kd[d]) return false;
    // 3D: both intermediate arrays (N0 x K1 x K2 and N0 x N1 x K2, times B)
    // fit in the coil-major buffer
    if (p->ndim == 3 && (int64_t)p->Nd[0] * (p->Kd[1] + p->Nd[1]) > (int64_t)p->Kd[0] * p->Kd[1])
        return false;
    // 32-bit batch and block indices in a pass
    return p->prodK * p->B < ((int64_t)1 << 31);
}

int cfft_init(nufft_plan_s* p) {
    if (!p->cfft) return NUFFT_OK;
    // twiddle tables exp(-2 pi i m / L) for every axis's length, from double
    std::vector<float2> h;
    for (int d = 0; d < p->ndim; ++d) {
        const int L = p->Kd[d];
        for (int m = 0; m < L; ++m) {
            const double ang = -2.0 * M_PI * (double)m / (double)L;
            h.push_back(make_float2((float)std::cos(ang), (float)std::sin(ang)));
        }
    }
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_cfft_tw, sizeof(float2) * h.size()));
    p->dev_bytes += sizeof(float2) * h.size();
    NUFFT_CUDA_TRY(cudaMemcpy(p->d_cfft_tw, h.data(), sizeof(float2) * h.size(),
                              cudaMemcpyHostToDevice));
    return NUFFT_OK;
}

void cfft_free(nufft_plan_s* p) {
    cudaFree(p->d_cfft_tw);
    p->d_cfft_tw = nullptr;
    p->cfft = false;
}

// image xx (Nd x B) -> spectrum k (Kd x B), through p->d_cm; dom_axis >= 0
// multiplies the image by -i (n_a - N_a/2) along that axis
int cfft_forward(nufft_plan_s* p, const float2* xx, bool apply_sn, int dom_axis, float2* k,
                 cudaStream_t s) {
    const int64_t B = p->B;
    const int* N = p->Nd;
    const int* K = p->Kd;
    const int nd = p->ndim, last = nd - 1;
    // the last axis: the image's rows -> mid (Nd[..last) x K[last] x B)
    float2* mid = p->d_cm;
    int64_t outer = 1;
    for (int d = 0; d < last; ++d) outer *= N[d];
    // 3D: mid2 (N0 x K1 x K2 x B) first in the buffer, mid1 (N0 x N1 x K2 x B) after it
    float2* mid2 = p->d_cm;
    float2* mid1 = (nd == 3) ? p->d_cm + (int64_t)N[0] * K[1] * K[2] * B : mid;
    CfftArgs a = pass_args(p, xx, mid1, last, (int64_t)N[last] * B, (int64_t)K[last] * B, B,
                           N[last], K[last]);
    a.apply_sn = apply_sn ? 1 : 0;
    if (dom_axis >= 0) {
        a.dom = (dom_axis == last) ? 2 : dom_axis;
        a.dom_half = 0.5f * (float)N[dom_axis];
    }
    NUFFT_TRY((run_len<false, 1>(K[last], a, outer, s)));
    if (nd == 3) {   // y: mid1[n0][n1][k2 b] -> mid2[n0][k1][k2 b]
        const int64_t in2 = (int64_t)K[2] * B;
        CfftArgs c = pass_args(p, mid1, mid2, 1, (int64_t)N[1] * in2, (int64_t)K[1] * in2, in2,
                               N[1], K[1]);
        NUFFT_TRY((run_len<false, 0>(K[1], c, N[0], s)));
    }
    // x: [n0][rest] -> k[k0][rest]
    const int64_t rest = p->prodK / K[0] * B;
    CfftArgs c = pass_args(p, nd == 3 ? mid2 : mid1, k, 0, 0, 0, rest, N[0], K[0]);
    return run_len<false, 0>(K[0], c, 1, s);
}

// spectrum k (Kd x B, read only) -> image xx (Nd x B): inverse transform,
// crop, x 1/prod(Kd), x sn when apply_sn, / sn when divide_sn.  With
// dscal, k is the 64-bit fixed-point sums of a deterministic gridding
// (2 x Kd x B, re and im), rounded by the first pass.
static int cfft_inverse_any(nufft_plan_s* p, const float2* k, const double* dscal, float2* xx,
                            bool apply_sn, bool divide_sn, cudaStream_t s) {
    const int64_t B = p->B;
    const int* N = p->Nd;
    const int* K = p->Kd;
    const int nd = p->ndim, last = nd - 1;
    float2* mid2 = p->d_cm;
    float2* mid1 = (nd == 3) ? p->d_cm + (int64_t)N[0] * K[1] * K[2] * B : p->d_cm;
    // x: k[k0][rest] -> [n0 < N0][rest]
    const int64_t rest = p->prodK / K[0] * B;
    CfftArgs c = pass_args(p, k, nd == 3 ? mid2 : mid1, 0, 0, 0, rest, K[0], N[0]);
    c.dscal = dscal;
    if (dscal)
        NUFFT_TRY((run_len<true, 3>(K[0], c, 1, s)));
    else
        NUFFT_TRY((run_len<true, 0>(K[0], c, 1, s)));
    if (nd == 3) {   // y: mid2[n0][k1][k2 b] -> mid1[n0][n1 < N1][k2 b]
        const int64_t in2 = (int64_t)K[2] * B;
        CfftArgs c2 = pass_args(p, mid2, mid1, 1, (int64_t)K[1] * in2, (int64_t)N[1] * in2, in2,
                                K[1], N[1]);
        NUFFT_TRY((run_len<true, 0>(K[1], c2, N[0], s)));
    }
    // the last axis: mid1 -> the image's rows, cropped and scaled
    int64_t outer = 1;
    for (int d = 0; d < last; ++d) outer *= N[d];
    CfftArgs a = pass_args(p, mid1, xx, last, (int64_t)K[last] * B, (int64_t)N[last] * B, B,
                           K[last], N[last]);
    a.apply_sn = apply_sn ? 1 : 0;
    a.divide_sn = divide_sn ? 1 : 0;
    a.norm = (float)(1.0 / (double)p->prodK);
    return run_len<true, 2>(K[last], a, outer, s);
}

int cfft_inverse(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn, bool divide_sn,
                 cudaStream_t s) {
    return cfft_inverse_any(p, k, nullptr, xx, apply_sn, divide_sn, s);
}

int cfft_inverse_fixed(nufft_plan_s* p, const unsigned long long* ig, const double* dscal,
                       float2* xx, bool apply_sn, bool divide_sn, cudaStream_t s) {
    return cfft_inverse_any(p, reinterpret_cast<const float2*>(ig), dscal, xx, apply_sn, divide_sn,
                            s);
}

}  // namespace nufft

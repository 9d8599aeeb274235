// Coil-batched FFT passes on coil-fastest layouts: the image <-> spectrum
// transforms of 2D plans of several coils (a multiple of 8) and one
// instance, with every Kd in {256, 384, 512, 640}.
//
// The reference's batch layout keeps the coil index fastest in the image,
// the spectrum and the samples (linalg/nufft_hsa.py:203-228).  These passes
// transform that layout in place of the coil-major copy, transposes and
// cuFFT calls: one pass per axis, each a set of L-point transforms along a
// strided axis whose batch (coils, or coils x cells) is contiguous.  A block
// takes 8 contiguous batch elements (64 bytes per row) and runs their 8
// transforms together: a mixed-radix Stockham FFT in three radix stages
// (640 = 10 x 8 x 8, 512 = 8 x 8 x 8, 384 = 6 x 8 x 8, 256 = 4 x 8 x 8),
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

struct CfftArgs {
    const float2* in;
    float2* out;
    int64_t in_so, in_sl;    // input strides (elements) of the outer and transform indices
    int64_t out_so, out_sl;  // output strides
    int inner;               // batch elements per (outer, index)
    int nchunk;              // blocks per outer index: ceil(inner / kCW)
    int lin, lout;           // inputs read (the rest are zero), outputs written
    const float2* tw;        // exp(-2 pi i m / L), m < L
    // image side: MODE 1 scales the input, MODE 2 the output (o = n0, l = n1)
    const float* sn_o;
    const float* sn_l;
    int apply_sn, divide_sn, dom_axis;
    float half_o, half_l;    // N0 / 2, N1 / 2 (the trajectory derivative's centre)
    float norm;
};

template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2* tw, int m) {
    const float2 v = tw[m];
    return INV ? make_float2(v.x, -v.y) : v;
}

template <int MODE>
__device__ __forceinline__ float2 pre_op(const CfftArgs& a, int o, int l, float2 v) {
    if constexpr (MODE == 1) {
        if (a.apply_sn) {
            const float sc = __ldg(a.sn_o + o) * __ldg(a.sn_l + l);
            v.x *= sc;
            v.y *= sc;
        }
        if (a.dom_axis >= 0) {   // x -i (n_a - N_a / 2)
            const float t = (a.dom_axis == 0) ? (float)o - a.half_o : (float)l - a.half_l;
            v = make_float2(t * v.y, -t * v.x);
        }
    }
    return v;
}

template <int MODE>
__device__ __forceinline__ float2 post_op(const CfftArgs& a, int o, int l, float2 v) {
    if constexpr (MODE == 2) {
        const float snv = __ldg(a.sn_o + o) * __ldg(a.sn_l + l);
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
    const bool ok = e < a.inner;
    const float2* __restrict__ in = a.in + o * a.in_so + e;
    float2* __restrict__ out = a.out + o * a.out_so + e;

    {   // stage 0: global -> shared (inputs past lin are zero)
        using S = typename P::S0;
        float2 v[R0];
        const bool act = j < S::NB;
        if (act) {
#pragma unroll
            for (int r = 0; r < R0; ++r) {
                const int l = S::in_index(j, r);
                v[r] = (ok && l < a.lin) ? pre_op<MODE>(a, o, l, __ldg(in + l * a.in_sl))
                                         : make_float2(0.f, 0.f);
            }
            cdft::dft<R0, INV>(v);
        }
        __syncthreads();   // the twiddle table is in place
        if (act) {
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
            if (ok) {
#pragma unroll
                for (int r = 0; r < R2; ++r) {
                    const int l = S::out_index(j, r);
                    if (l < a.lout) out[l * a.out_sl] = post_op<MODE>(a, o, l, v[r]);
                }
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
    if (blocks > 0) kern<<<(unsigned)blocks, P::THREADS, P::SMEM, s>>>(a);
    return check_launch("cfft_pass_kernel");
}

template <bool INV, int MODE>
int run_len(int L, const CfftArgs& a, int64_t outer, cudaStream_t s) {
    switch (L) {
        case 640: return run_pass<640, 10, 8, 8, INV, MODE>(a, outer, s);
        case 512: return run_pass<512, 8, 8, 8, INV, MODE>(a, outer, s);
        case 384: return run_pass<384, 6, 8, 8, INV, MODE>(a, outer, s);
        case 256: return run_pass<256, 4, 8, 8, INV, MODE>(a, outer, s);
        default:
            set_error("cfft: unsupported transform length");
            return NUFFT_EUNSUPPORTED;
    }
}

bool length_ok(int L) { return L == 256 || L == 384 || L == 512 || L == 640; }

CfftArgs image_args(const nufft_plan_s* p) {
    CfftArgs a{};
    a.sn_o = p->d_snd;
    a.sn_l = p->d_snd + p->Nd[0];
    a.half_o = 0.5f * (float)p->Nd[0];
    a.half_l = 0.5f * (float)p->Nd[1];
    a.dom_axis = -1;
    a.norm = 1.f;
    return a;
}

}  // namespace

bool cfft_eligible(const nufft_plan_s* p) {
    if (p->flags & NUFFT_FLAG_CUFFT) return false;
    if (p->ndim != 2 || p->ninst != 1 || p->B < 8 || p->B % kCW != 0) return false;
    if (!length_ok(p->Kd[0]) || !length_ok(p->Kd[1])) return false;
    // batch chunks of kCW columns over K1 B, and int32 indices in a pass
    return (int64_t)p->Kd[0] * p->Kd[1] * p->B < ((int64_t)1 << 31);
}

int cfft_init(nufft_plan_s* p) {
    if (!p->cfft) return NUFFT_OK;
    // twiddle tables exp(-2 pi i m / L) for both axes' lengths, from double
    const int L0 = p->Kd[0], L1 = p->Kd[1];
    std::vector<float2> h((size_t)L0 + L1);
    for (int d = 0; d < 2; ++d) {
        const int L = p->Kd[d];
        float2* t = h.data() + (d == 0 ? 0 : L0);
        for (int m = 0; m < L; ++m) {
            const double ang = -2.0 * M_PI * (double)m / (double)L;
            t[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
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

// image xx (N0 x N1 x B) -> spectrum k (K0 x K1 x B), through p->d_cm
int cfft_forward(nufft_plan_s* p, const float2* xx, bool apply_sn, int dom_axis, float2* k,
                 cudaStream_t s) {
    const int B = p->B, N0 = p->Nd[0], N1 = p->Nd[1], K0 = p->Kd[0], K1 = p->Kd[1];
    float2* mid = p->d_cm;   // N0 x K1 x B
    CfftArgs a = image_args(p);
    // rows: x[n0][n1][b] -> mid[n0][k1][b]
    a.in = xx;
    a.out = mid;
    a.in_so = (int64_t)N1 * B;
    a.in_sl = B;
    a.out_so = (int64_t)K1 * B;
    a.out_sl = B;
    a.inner = B;
    a.nchunk = (B + kCW - 1) / kCW;
    a.lin = N1;
    a.lout = K1;
    a.tw = p->d_cfft_tw + K0;
    a.apply_sn = apply_sn ? 1 : 0;
    a.dom_axis = dom_axis;
    NUFFT_TRY((run_len<false, 1>(K1, a, N0, s)));
    // columns: mid[n0][k1 b] -> k[k0][k1 b]
    CfftArgs c = image_args(p);
    c.in = mid;
    c.out = k;
    c.in_so = c.out_so = 0;
    c.in_sl = c.out_sl = (int64_t)K1 * B;
    c.inner = K1 * B;
    c.nchunk = (c.inner + kCW - 1) / kCW;
    c.lin = N0;
    c.lout = K0;
    c.tw = p->d_cfft_tw;
    return run_len<false, 0>(K0, c, 1, s);
}

// spectrum k (K0 x K1 x B, read only) -> image xx (N0 x N1 x B): inverse
// transform, crop, x 1/prod(Kd), x sn when apply_sn, / sn when divide_sn
int cfft_inverse(nufft_plan_s* p, const float2* k, float2* xx, bool apply_sn, bool divide_sn,
                 cudaStream_t s) {
    const int B = p->B, N0 = p->Nd[0], N1 = p->Nd[1], K0 = p->Kd[0], K1 = p->Kd[1];
    float2* mid = p->d_cm;
    // columns: k[k0][k1 b] -> mid[n0 < N0][k1 b]
    CfftArgs c = image_args(p);
    c.in = k;
    c.out = mid;
    c.in_so = c.out_so = 0;
    c.in_sl = c.out_sl = (int64_t)K1 * B;
    c.inner = K1 * B;
    c.nchunk = (c.inner + kCW - 1) / kCW;
    c.lin = K0;
    c.lout = N0;
    c.tw = p->d_cfft_tw;
    NUFFT_TRY((run_len<true, 0>(K0, c, 1, s)));
    // rows: mid[n0][k1][b] -> x[n0][n1 < N1][b]
    CfftArgs a = image_args(p);
    a.in = mid;
    a.out = xx;
    a.in_so = (int64_t)K1 * B;
    a.in_sl = B;
    a.out_so = (int64_t)N1 * B;
    a.out_sl = B;
    a.inner = B;
    a.nchunk = (B + kCW - 1) / kCW;
    a.lin = K1;
    a.lout = N1;
    a.tw = p->d_cfft_tw + K0;
    a.apply_sn = apply_sn ? 1 : 0;
    a.divide_sn = divide_sn ? 1 : 0;
    a.norm = (float)(1.0 / (double)p->prodK);
    return run_len<true, 2>(K1, a, N0, s);
}

}  // namespace nufft

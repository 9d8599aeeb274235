// Pruned power-of-two FFTs of one coil and one instance (2D and 3D plans
// whose every Kd is a power of two, 16 .. 4096), used when the plan asks for
// them (NUFFT_FLAG_OWN_FFT) and, unless it asks for cuFFT (NUFFT_FLAG_CUFFT),
// by default where every pass is a 256-point one; plans otherwise run cuFFT.
//
// The reference's xx2k zero-pads the image into the Kd array and runs numpy's
// fftn over it (_xx2k_cpu, nufft/_nufft_class_methods_cpu.py:232-249); k2xx
// runs ifftn and crops the first Nd entries of every axis (_k2xx_cpu,
// :316-329).  Here the transform runs one axis at a time and neither reads
// nor writes the padding:
//
//   forward  x (N0,N1,N2) --last axis, x sn--> T1 (N0,N1,K2)
//                         --middle axis------> T2 (N0,K1,K2)
//                         --first axis-------> k  (K0,K1,K2)
//   inverse  k --first axis, keep N0--> T2 --middle, keep N1--> T1
//              --last axis, keep N2, / prod(Kd), x or / sn--> x
//
// (2D: the same with the middle axis as the first, and no third pass.)  Each
// pass takes its columns in tiles of C columns x K entries (C K = 4096, 16
// entries per thread) and runs a Stockham autosort FFT on every column with
// radix-16 butterflies held in registers (a radix-2/4/8 stage last when
// log2 K is not a multiple of 4; the stage structure of Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors", SC
// 2008).  The first stage reads straight from global memory and the last
// writes straight to it, so a 256-point axis makes one round trip through
// shared memory; the shared column is padded by one entry per 16 so the
// butterflies' strided writes fall in distinct banks.  Entries past the input
// extent are zero in registers and never loaded; entries past the output
// extent are never stored.  At Kd = 2 Nd this moves 352 MB per 256^3
// transform instead of the ~570 MB of the zero-padded cuFFT passes.  These
// general passes are bound by instruction issue (~3 TB/s: 0.125 / 0.128 ms
// forward / inverse at 256^3 against cuFFT's 0.110 / ~0.105 ms; 0.019 /
// 0.019 against 0.015 / 0.020 ms at 512^2); 256-point passes run
// pfft256_kernel instead, with every size fixed at compile time (0.077 /
// 0.091 ms at 256^3 against 0.111 / 0.146 for the cuFFT stages with their
// pad and crop), which is why those plans take the own passes by default.
// T1 and T2 live in the plan's d_padin / d_slabout buffers.
#include "nufft_internal.cuh"

#include <cmath>

namespace nufft {

namespace {

constexpr int kTileElems = 4096;   // largest tile of a contiguous pass: C x K entries
constexpr int kPassThreads = 256;  // its threads
constexpr int kPassBlocks = 2;     // resident 256-thread blocks per SM (128 registers)
// (strided passes with twice the columns in one 512-thread block per SM
// measured slower: 0.131 / 0.140 ms against 0.125 / 0.128 ms at 256^3)
template <bool CONTIG> constexpr int tile_elems() { return kTileElems; }
template <bool CONTIG> constexpr int tile_threads() { return kPassThreads; }
template <bool CONTIG> constexpr int tile_blocks() { return kPassBlocks; }
constexpr int kPer = 16;           // entries per thread in every stage (C K / 16 threads)
constexpr int kMaxStages = 3;      // K <= 4096 = 16^3

struct PfftPass {
    int K, lgK;          // transform length along the axis and its log2
    int C, lgC;          // columns per tile (a power of two)
    int P;               // shared-memory stride of a column (odd, >= padded K)
    int nstage;          // Stockham stages and their radices (16, then 2/4/8)
    int radix[kMaxStages];
    int n_in, n_out;     // entries read (the rest are zero) / written per column
    int64_t ncol;        // columns per batch
    int64_t nbatch;      // batches
    int64_t in_b, in_c, in_i;     // input element strides: batch, column, axis entry
    int64_t out_b, out_c, out_i;  // output element strides
    // stage s >= 1 twiddles W_{Ns R}^{r k} = exp(-2 pi i r k / (Ns R)) at
    // [k R + r] (Ns: product of the earlier radices; stage 0 has none)
    const float2* stw[kMaxStages];
    int inverse;         // 0: exp(-2 pi i ...) (numpy fft), 1: exp(+2 pi i ...)
    // image scaling of the contiguous passes, whose columns are image rows:
    // row r has lead factor sa[r / nb] * sb[r % nb] (a null pointer counts
    // as 1) and entry i the factor sl[i]
    const float* sa;
    const float* sb;
    int nb;
    const float* sl;
    int scale_in;        // forward: input x sn
    int scale_out;       // inverse: 0 none, 1 x sn, 2 / sn; always x norm
    float norm;
};

const float* sn_ptr(const nufft_plan_s* p, int axis) {
    const float* s = p->d_snd;
    for (int d = 0; d < axis; ++d) s += p->Nd[d];
    return s;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * w, or a * conj(w) for the inverse transform
__device__ __forceinline__ float2 cmul_tw(float2 a, float2 w, bool inv) {
    return cmul(a, inv ? make_float2(w.x, -w.y) : w);
}

// exp(-+2 pi i m / 16), m = 0 .. 15 (cos and sin of multiples of pi / 8);
// the index is a compile-time constant after unrolling
__device__ __forceinline__ float2 w16(int m, bool inv) {
    constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f, c2 = 0.70710678118654752f;
    const float cs[16] = {1.f, c1, c2, s1, 0.f, -s1, -c2, -c1, -1.f, -c1, -c2, -s1, 0.f, s1, c2, c1};
    const float sn[16] = {0.f, s1, c2, c1, 1.f, c1, c2, s1, 0.f, -s1, -c2, -c1, -1.f, -c1, -c2, -s1};
    return make_float2(cs[m & 15], inv ? sn[m & 15] : -sn[m & 15]);
}

// 4-point DFT in place; the +-i of the odd outputs follows the sign
__device__ __forceinline__ void dft4(float2& a, float2& b, float2& c, float2& d, bool inv) {
    const float2 s02 = cadd(a, c), d02 = csub(a, c), s13 = cadd(b, d), d13 = csub(b, d);
    const float2 mi = inv ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
    a = cadd(s02, s13);
    b = cadd(d02, mi);
    c = csub(s02, s13);
    d = csub(d02, mi);
}

// R-point DFT of v[o .. o + R) in place: V[q] = sum_r v[r] exp(-+2 pi i r q / R).
// R = 8: radix 4 x 2; R = 16: radix 4 x 4 (r = n2 + 4 n1, q = q1 + 4 q2).
template <int R>
__device__ __forceinline__ void dftR(float2 (&v)[kPer], int o, bool inv) {
    if (R == 2) {
        const float2 a = v[o], b = v[o + 1];
        v[o] = cadd(a, b);
        v[o + 1] = csub(a, b);
    } else if (R == 4) {
        dft4(v[o], v[o + 1], v[o + 2], v[o + 3], inv);
    } else if (R == 8) {
        float2 y[8];
#pragma unroll
        for (int n2 = 0; n2 < 2; ++n2) {
            float2 a = v[o + n2], b = v[o + n2 + 2], c = v[o + n2 + 4], d = v[o + n2 + 6];
            dft4(a, b, c, d, inv);
            y[n2 * 4 + 0] = a; y[n2 * 4 + 1] = b; y[n2 * 4 + 2] = c; y[n2 * 4 + 3] = d;
        }
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) {
            const float2 y0 = y[q1], y1 = cmul(y[4 + q1], w16(2 * q1, inv));
            v[o + q1] = cadd(y0, y1);
            v[o + q1 + 4] = csub(y0, y1);
        }
    } else {
        float2 y[16];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            float2 a = v[o + n2], b = v[o + n2 + 4], c = v[o + n2 + 8], d = v[o + n2 + 12];
            dft4(a, b, c, d, inv);
            y[n2 * 4 + 0] = a;
            y[n2 * 4 + 1] = cmul(b, w16(n2, inv));
            y[n2 * 4 + 2] = cmul(c, w16(2 * n2, inv));
            y[n2 * 4 + 3] = cmul(d, w16(3 * n2, inv));
        }
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) {
            float2 a = y[q1], b = y[4 + q1], c = y[8 + q1], d = y[12 + q1];
            dft4(a, b, c, d, inv);
            v[o + q1] = a; v[o + q1 + 4] = b; v[o + q1 + 8] = c; v[o + q1 + 12] = d;
        }
    }
}

__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }

__device__ __forceinline__ float row_lead(const PfftPass& q, int r) {
    float s = 1.f;
    if (q.sa) s *= __ldg(q.sa + r / q.nb);
    if (q.sb) s *= __ldg(q.sb + r % q.nb);
    return s;
}

// One tile's position.
struct TilePos {
    int64_t bt, c0;
    int cn;
};

// Butterfly b of a stage with radix R -> (column c, butterfly j).  CONTIG:
// j fastest across threads (the axis is contiguous in global memory); else c
// fastest (the columns are).
template <bool CONTIG>
__device__ __forceinline__ void butterfly_of(const PfftPass& q, int lgR, int b, int& c, int& j) {
    if (CONTIG) {
        const int lgJ = q.lgK - lgR;
        c = b >> lgJ;
        j = b & ((1 << lgJ) - 1);
    } else {
        c = b & (q.C - 1);
        j = b >> q.lgC;
    }
}

// The first stage's inputs of a tile (its radix is 16: every K >= 16): the
// 16 entries of each thread's butterfly, zero past the input extent.  Issued
// for the next tile while the current one finishes, so that the loads'
// latency overlaps its remaining stages.
template <bool CONTIG>
__device__ __forceinline__ void load_first(const PfftPass& q, const TilePos& tp,
                                           const float2* __restrict__ in, float2 (&v)[kPer]) {
    const int stride = q.K >> 4;
    int c, j;
    butterfly_of<CONTIG>(q, 4, threadIdx.x, c, j);
    const float2* sp = in + tp.bt * q.in_b + (tp.c0 + c) * q.in_c + (int64_t)j * q.in_i;
    const int64_t dr = (int64_t)stride * q.in_i;
    const bool col = c < tp.cn;
#pragma unroll
    for (int r = 0; r < kPer; ++r)
        v[r] = (col && j + r * stride < q.n_in) ? __ldg(sp + r * dr) : make_float2(0.f, 0.f);
}

// One Stockham stage with radix R over the tile: every one of the C K / 16
// threads takes kPer / R butterflies.  The first stage takes the inputs that
// load_first brought into `pre` (x sn on the forward contiguous pass), the
// last writes global memory (crop, / prod(Kd) and sn on the inverse
// contiguous pass); the others read and write the shared columns in place,
// with a barrier between all reads and the first write.
template <int R, bool CONTIG, bool INV>
__device__ __forceinline__ void pfft_stage(const PfftPass& q, const TilePos& tp, int Ns,
                                           bool first, bool last, const float2* __restrict__ stw,
                                           float2* sm, const float* s_lead,
                                           const float2 (&pre)[kPer], float2* __restrict__ out) {
    constexpr int NB = kPer / R;
    constexpr int lgR = (R == 2) ? 1 : (R == 4) ? 2 : (R == 8) ? 3 : 4;
    const int stride = q.K >> lgR;   // K / R
    constexpr bool inv = INV;
    float2 v[kPer];
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        int c, j;
        butterfly_of<CONTIG>(q, lgR, threadIdx.x + m * blockDim.x, c, j);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = j + r * stride;
            if (first) {   // R == 16, NB == 1
                float2 x = pre[r];
                if (CONTIG && q.scale_in && c < tp.cn && i < q.n_in) {
                    const float sv = s_lead[c] * __ldg(q.sl + i);
                    x.x *= sv;
                    x.y *= sv;
                }
                v[m * R + r] = x;
            } else {
                v[m * R + r] = sm[c * q.P + padi(i)];
            }
        }
    }
    if (!first) __syncthreads();   // every read of this stage before any write
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        int c, j;
        butterfly_of<CONTIG>(q, lgR, threadIdx.x + m * blockDim.x, c, j);
        const int k = j & (Ns - 1);
        if (Ns > 1) {   // this butterfly's R twiddles, contiguous: R / 2 16-byte loads
            const float4* t4 = reinterpret_cast<const float4*>(stw + k * R);
#pragma unroll
            for (int h = 0; h < R / 2; ++h) {
                const float4 w = __ldg(t4 + h);
                if (h > 0) v[m * R + 2 * h] = cmul_tw(v[m * R + 2 * h], make_float2(w.x, w.y), inv);
                v[m * R + 2 * h + 1] = cmul_tw(v[m * R + 2 * h + 1], make_float2(w.z, w.w), inv);
            }
        }
        dftR<R>(v, m * R, inv);
        const int o0 = (j - k) * R + k;
        if (last) {
            float2* dp = out + tp.bt * q.out_b + (tp.c0 + c) * q.out_c + (int64_t)o0 * q.out_i;
            const int64_t ds = (int64_t)Ns * q.out_i;
            if (c < tp.cn) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int o = o0 + r * Ns;
                    if (o >= q.n_out) continue;
                    float2 x = v[m * R + r];
                    if (CONTIG) {
                        float sc = q.norm;
                        if (q.scale_out) {
                            const float snv = s_lead[c] * __ldg(q.sl + o);
                            if (q.scale_out == 1) sc *= snv;
                            x.x *= sc;
                            x.y *= sc;
                            if (q.scale_out == 2) {
                                x.x /= snv;
                                x.y /= snv;
                            }
                        } else {
                            x.x *= sc;
                            x.y *= sc;
                        }
                    }
                    dp[r * ds] = x;
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) sm[c * q.P + padi(o0 + r * Ns)] = v[m * R + r];
        }
    }
    if (!last) __syncthreads();   // the next stage reads what this one wrote
}

template <bool CONTIG, bool INV>
__device__ __forceinline__ void pfft_stage_r(const PfftPass& q, const TilePos& tp, int s, int Ns,
                                             float2* sm, const float* s_lead,
                                             const float2 (&pre)[kPer], float2* __restrict__ out) {
    const bool first = (s == 0), last = (s == q.nstage - 1);
    const float2* stw = q.stw[s];
    switch (q.radix[s]) {
        case 16: pfft_stage<16, CONTIG, INV>(q, tp, Ns, first, last, stw, sm, s_lead, pre, out); break;
        case 8: pfft_stage<8, CONTIG, INV>(q, tp, Ns, first, last, stw, sm, s_lead, pre, out); break;
        case 4: pfft_stage<4, CONTIG, INV>(q, tp, Ns, first, last, stw, sm, s_lead, pre, out); break;
        default: pfft_stage<2, CONTIG, INV>(q, tp, Ns, first, last, stw, sm, s_lead, pre, out); break;
    }
}

__device__ __forceinline__ TilePos tile_pos(const PfftPass& q, int64_t t, int64_t tiles_per_batch) {
    TilePos tp;
    tp.bt = t / tiles_per_batch;
    tp.c0 = (t - tp.bt * tiles_per_batch) << q.lgC;
    const int64_t rest = q.ncol - tp.c0;
    tp.cn = rest < (int64_t)q.C ? (int)rest : q.C;
    return tp;
}

// One pass.  CONTIG: the transform axis is contiguous in memory (columns are
// rows); else the columns are contiguous.  Shared memory: C padded columns
// P entries apart (P odd, so the column-crossing accesses of the strided
// passes fall in distinct banks), and the per-row factors of the contiguous
// passes.
template <bool CONTIG, bool INV>
__global__ void __launch_bounds__(tile_threads<CONTIG>(), tile_blocks<CONTIG>()) pfft_pass_kernel(PfftPass q,
                                                                   const float2* __restrict__ in,
                                                                   float2* __restrict__ out) {
    extern __shared__ float2 pf_smem[];
    __shared__ float s_lead[kTileElems / 16];   // C <= 256
    const int64_t tiles_per_batch = (q.ncol + q.C - 1) >> q.lgC;
    const int64_t ntiles = tiles_per_batch * q.nbatch;
    const bool scaled = CONTIG && (q.scale_in || q.scale_out);
    float2 pre[kPer];
    if ((int64_t)blockIdx.x < ntiles) load_first<CONTIG>(q, tile_pos(q, blockIdx.x, tiles_per_batch), in, pre);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TilePos tp = tile_pos(q, t, tiles_per_batch);
        if (scaled) {   // image rows < 2^31
            for (int c = threadIdx.x; c < tp.cn; c += blockDim.x)
                s_lead[c] = row_lead(q, (int)(tp.c0 + c));
            __syncthreads();
        }
        int Ns = 1;
        for (int s = 0; s < q.nstage; ++s) {
            pfft_stage_r<CONTIG, INV>(q, tp, s, Ns, pf_smem, s_lead, pre, out);
            Ns *= q.radix[s];
            if (s == 0 && t + gridDim.x < ntiles)   // the next tile's inputs, in flight meanwhile
                load_first<CONTIG>(q, tile_pos(q, t + gridDim.x, tiles_per_batch), in, pre);
        }
        __syncthreads();   // the next tile reuses the columns and the row factors
    }
}

// 256-point passes (every axis of a 256^D grid): 16 columns per 256-thread
// block, 16 entries per thread, the 16 x 16 decomposition with all sizes
// fixed at compile time: entry n = t + 16 j; a 16-point DFT over j in
// registers (index k1), the twiddle W256^(t k1) from a shared table, one
// exchange through shared memory (padded so both sides are free of bank
// conflicts), a 16-point DFT over t (index k2): X[k1 + 16 k2].  NIN / NOUT:
// entries read / written per column (128 where the other half is the zero
// padding or is cropped away).  CONTIG: the lanes run along the column (the
// transform axis is contiguous); else across 16 adjacent columns.
template <bool CONTIG, bool INV, int NIN, int NOUT>
__device__ __forceinline__ void pfft256_body(const PfftPass& q, const float2* __restrict__ in,
                                             float2* __restrict__ out) {
    __shared__ float2 sx[16 * 257];   // entry (k1, column, t), k1-major, 257 apart
    __shared__ float2 stw[256];       // W256^(t k1) at [k1 16 + t]
    {
        const int k1 = threadIdx.x >> 4, t = threadIdx.x & 15;
        float sn, cs;
        sincospif(-(float)(t * k1) / 128.f, &sn, &cs);
        stw[threadIdx.x] = make_float2(cs, INV ? -sn : sn);
    }
    __syncthreads();
    const int lo = threadIdx.x & 15, hi = threadIdx.x >> 4;
    const int t = CONTIG ? lo : hi;    // first stage: this thread's subsequence
    const int cl = CONTIG ? hi : lo;   // its column within the tile
    const int k1 = CONTIG ? lo : hi;   // second stage: its frequency k1
    const int64_t per_batch = (q.ncol + 15) >> 4;
    const int64_t ntiles = per_batch * q.nbatch;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t bt = tile / per_batch;
        const int64_t col = ((tile - bt * per_batch) << 4) + cl;
        const bool live = col < q.ncol;
        float lead = 1.f;
        if (CONTIG && (q.scale_in || q.scale_out) && live) lead = row_lead(q, (int)col);
        float2 v[16];
        const float2* ip = in + bt * q.in_b + col * q.in_c;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int i = t + 16 * j;
            float2 x = make_float2(0.f, 0.f);
            if (j < NIN / 16 && live) {
                x = __ldg(ip + (int64_t)i * q.in_i);
                if (CONTIG && q.scale_in) {
                    const float sv = lead * __ldg(q.sl + i);
                    x.x *= sv;
                    x.y *= sv;
                }
            }
            v[j] = x;
        }
        dftR<16>(v, 0, INV);
#pragma unroll
        for (int k = 1; k < 16; ++k) v[k] = cmul(v[k], stw[k * 16 + t]);
#pragma unroll
        for (int k = 0; k < 16; ++k) sx[k * 257 + (CONTIG ? cl * 16 + t : t * 16 + cl)] = v[k];
        __syncthreads();
#pragma unroll
        for (int tt = 0; tt < 16; ++tt) v[tt] = sx[k1 * 257 + (CONTIG ? cl * 16 + tt : tt * 16 + cl)];
        __syncthreads();   // the next tile's writes come after every read
        dftR<16>(v, 0, INV);
        if (live) {
            float2* op = out + bt * q.out_b + col * q.out_c;
#pragma unroll
            for (int k2 = 0; k2 < NOUT / 16; ++k2) {
                const int o = k1 + 16 * k2;
                float2 x = v[k2];
                if (CONTIG) {
                    float sc = q.norm;
                    if (q.scale_out) {
                        const float snv = lead * __ldg(q.sl + o);
                        if (q.scale_out == 1) sc *= snv;
                        x.x *= sc;
                        x.y *= sc;
                        if (q.scale_out == 2) {
                            x.x /= snv;
                            x.y /= snv;
                        }
                    } else {
                        x.x *= sc;
                        x.y *= sc;
                    }
                }
                op[(int64_t)o * q.out_i] = x;
            }
        }
    }
}

// Passes reading every entry hold four blocks per SM with a 64-register cap
// (256^3 inverse 0.092 -> 0.078 ms); the half-input passes fit four blocks
// without it and spill under it (forward 0.077 -> 0.083 ms).
template <bool CONTIG, bool INV, int NOUT>
__global__ void __launch_bounds__(256) pfft256_half_kernel(PfftPass q, const float2* __restrict__ in,
                                                           float2* __restrict__ out) {
    pfft256_body<CONTIG, INV, 128, NOUT>(q, in, out);
}
template <bool CONTIG, bool INV, int NOUT>
__global__ void __launch_bounds__(256, 4) pfft256_full_kernel(PfftPass q, const float2* __restrict__ in,
                                                              float2* __restrict__ out) {
    pfft256_body<CONTIG, INV, 256, NOUT>(q, in, out);
}

template <bool CONTIG, bool INV, int NIN, int NOUT>
int run_pass256(const nufft_plan_s* p, const PfftPass& q, const float2* in, float2* out,
                cudaStream_t s) {
    const int64_t tiles = ((q.ncol + 15) / 16) * q.nbatch;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)p->num_sms * 4));
    if constexpr (NIN == 256)
        pfft256_full_kernel<CONTIG, INV, NOUT><<<blocks, 256, 0, s>>>(q, in, out);
    else
        pfft256_half_kernel<CONTIG, INV, NOUT><<<blocks, 256, 0, s>>>(q, in, out);
    return check_launch("pfft256 pass");
}

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

// Radices of the Stockham stages of a K-point transform: 16s, then 2, 4 or 8.
int radix_plan(int K, int (&radix)[kMaxStages]) {
    int n = 0;
    for (int rem = K; rem > 1;) {
        const int r = std::min(rem, 16);
        radix[n++] = r;
        rem /= r;
    }
    return n;
}

PfftPass base_pass(const nufft_plan_s* p, int axis, bool inverse) {
    PfftPass q{};
    q.K = p->Kd[axis];
    q.lgK = ilog2(q.K);
    q.C = std::max(1, kTileElems / q.K);   // narrowed by fit_tiles
    q.lgC = ilog2(q.C);
    q.P = (q.K + q.K / 16) | 1;
    q.nstage = radix_plan(q.K, q.radix);
    for (int s = 0; s < kMaxStages; ++s)
        q.stw[s] = (s > 0 && s < q.nstage) ? p->d_pfft_tw + p->pfft_tw_off[axis][s] : nullptr;
    q.inverse = inverse ? 1 : 0;
    q.nb = 1;
    q.norm = 1.f;
    return q;
}

// Narrow the tiles (fewer columns, C K / 16 threads down to 64) until the
// pass has at least four tiles per SM: small grids (512^2) otherwise leave
// most SMs idle.
void fit_tiles(const nufft_plan_s* p, PfftPass& q, int tile) {
    q.C = std::max(1, tile / q.K);
    q.lgC = ilog2(q.C);
    const int64_t want = 4 * (int64_t)std::max(p->num_sms, 1);
    while (q.C > 1 && (int64_t)q.C * q.K > 1024 &&
           ((q.ncol + q.C - 1) / q.C) * q.nbatch < want) {
        q.C >>= 1;
        --q.lgC;
    }
}

template <bool CONTIG, bool INV>
int run_pass_dir(const nufft_plan_s* p, PfftPass q, const float2* in, float2* out,
                 cudaStream_t s) {
    fit_tiles(p, q, tile_elems<CONTIG>());
    const int threads = q.C * q.K / kPer;                      // 64 .. 256
    const size_t smem = sizeof(float2) * (size_t)q.C * q.P;   // <= 36,872 B
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(pfft_pass_kernel<CONTIG, INV>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("pfft: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
    }
    const int64_t tiles = ((q.ncol + q.C - 1) / q.C) * q.nbatch;
    const int per_sm = tile_blocks<CONTIG>() * (tile_threads<CONTIG>() / threads);   // resident per SM
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)p->num_sms * per_sm));
    pfft_pass_kernel<CONTIG, INV><<<blocks, threads, smem, s>>>(q, in, out);
    return check_launch(CONTIG ? "pfft_pass_kernel<contig>" : "pfft_pass_kernel<strided>");
}

template <bool CONTIG>
int run_pass(const nufft_plan_s* p, const PfftPass& q, const float2* in, float2* out,
             cudaStream_t s) {
    if (q.K == 256 && (q.n_in == 128 || q.n_in == 256) && (q.n_out == 128 || q.n_out == 256)) {
        const bool hi_in = q.n_in == 256, hi_out = q.n_out == 256;
        if (q.inverse) {
            if (hi_in && hi_out) return run_pass256<CONTIG, true, 256, 256>(p, q, in, out, s);
            if (hi_in) return run_pass256<CONTIG, true, 256, 128>(p, q, in, out, s);
            if (hi_out) return run_pass256<CONTIG, true, 128, 256>(p, q, in, out, s);
            return run_pass256<CONTIG, true, 128, 128>(p, q, in, out, s);
        }
        if (hi_in && hi_out) return run_pass256<CONTIG, false, 256, 256>(p, q, in, out, s);
        if (hi_in) return run_pass256<CONTIG, false, 256, 128>(p, q, in, out, s);
        if (hi_out) return run_pass256<CONTIG, false, 128, 256>(p, q, in, out, s);
        return run_pass256<CONTIG, false, 128, 128>(p, q, in, out, s);
    }
    return q.inverse ? run_pass_dir<CONTIG, true>(p, q, in, out, s)
                     : run_pass_dir<CONTIG, false>(p, q, in, out, s);
}

}  // namespace

// Own passes: asked for (NUFFT_FLAG_OWN_FFT), or by default where every pass
// is a 256-point one (every Kd 256, every Nd 128 or 256: 3D 128^3 -> 256^3
// xx2k 0.077 / k2xx 0.091 ms against cuFFT's 0.111 / 0.146 ms); never with
// NUFFT_FLAG_CUFFT.
bool pfft_eligible(const nufft_plan_s* p) {
    if (p->flags & NUFFT_FLAG_CUFFT) return false;
    if (p->B != 1 || p->ninst != 1 || p->ndim < 2) return false;
    bool all256 = true;
    for (int d = 0; d < p->ndim; ++d) {
        const int K = p->Kd[d];
        if (K < 16 || K > 4096 || (K & (K - 1)) != 0 || p->Nd[d] > K) return false;
        all256 = all256 && K == 256 && (p->Nd[d] == 128 || p->Nd[d] == 256);
    }
    return (p->flags & NUFFT_FLAG_OWN_FFT) || all256;
}

int pfft_init(nufft_plan_s* p) {
    p->pfft = false;
    if (!pfft_eligible(p) || !p->d_padin || !p->d_slabout) return NUFFT_OK;
    // stage s >= 1 of each axis: W_{Ns R}^{r k} at [k R + r], in double then
    // rounded (every table has an even length, so every table and every
    // butterfly's run of R twiddles starts on 16 bytes)
    std::vector<float2> h;
    for (int d = 0; d < p->ndim; ++d) {
        int radix[kMaxStages];
        const int ns = radix_plan(p->Kd[d], radix);
        int Ns = 1;
        for (int st = 0; st < ns; ++st) {
            const int R = radix[st];
            p->pfft_tw_off[d][st] = (int)h.size();
            if (st > 0) {
                for (int k = 0; k < Ns; ++k)
                    for (int r = 0; r < R; ++r) {
                        const double a = -2.0 * M_PI * (double)(r * k) / (double)(Ns * R);
                        h.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
                    }
            }
            Ns *= R;
        }
    }
    const size_t n = std::max<size_t>(h.size(), 2);
    h.resize(n, make_float2(1.f, 0.f));
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_pfft_tw, sizeof(float2) * n));
    NUFFT_CUDA_TRY(cudaMemcpy(p->d_pfft_tw, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    p->dev_bytes += sizeof(float2) * n;
    p->pfft = true;
    return NUFFT_OK;
}

void pfft_free(nufft_plan_s* p) {
    cudaFree(p->d_pfft_tw);
    p->d_pfft_tw = nullptr;
    p->pfft = false;
}

// x (Nd, x sn when apply_sn) -> k (Kd): the forward passes above.
int pfft_forward(nufft_plan_s* p, const float2* x, bool apply_sn, float2* k, cudaStream_t s) {
    const int nd = p->ndim;
    const int N0 = p->Nd[0], N1 = p->Nd[1];
    const int K0 = p->Kd[0], K1 = p->Kd[1];
    const int last = nd - 1;
    const int NL = p->Nd[last], KL = p->Kd[last];
    float2* t1 = p->d_padin;
    // last axis: rows of the image -> T1 (rows x KL)
    PfftPass a = base_pass(p, last, false);
    a.n_in = NL;
    a.n_out = KL;
    a.ncol = (nd == 3) ? (int64_t)N0 * N1 : N0;
    a.nbatch = 1;
    a.in_c = NL; a.in_i = 1;
    a.out_c = KL; a.out_i = 1;
    if (apply_sn) {
        a.scale_in = 1;
        a.sa = (nd == 3) ? sn_ptr(p, 0) : nullptr;
        a.sb = (nd == 3) ? sn_ptr(p, 1) : sn_ptr(p, 0);
        a.nb = (nd == 3) ? N1 : N0;
        a.sl = sn_ptr(p, last);
    }
    NUFFT_TRY(run_pass<true>(p, a, x, t1, s));
    if (nd == 2) {
        // first axis: T1 (N0 x K1) -> k (K0 x K1), columns contiguous
        PfftPass b = base_pass(p, 0, false);
        b.n_in = N0; b.n_out = K0;
        b.ncol = K1; b.nbatch = 1;
        b.in_c = 1; b.in_i = K1;
        b.out_c = 1; b.out_i = K1;
        return run_pass<false>(p, b, t1, k, s);
    }
    const int K2 = p->Kd[2];
    float2* t2 = p->d_slabout;
    // middle axis: T1 (N0, N1, K2) -> T2 (N0, K1, K2), one batch per x
    PfftPass b = base_pass(p, 1, false);
    b.n_in = N1; b.n_out = K1;
    b.ncol = K2; b.nbatch = N0;
    b.in_b = (int64_t)N1 * K2; b.in_c = 1; b.in_i = K2;
    b.out_b = (int64_t)K1 * K2; b.out_c = 1; b.out_i = K2;
    NUFFT_TRY(run_pass<false>(p, b, t1, t2, s));
    // first axis: T2 (N0, K1 K2) -> k (K0, K1 K2)
    PfftPass c = base_pass(p, 0, false);
    c.n_in = N0; c.n_out = K0;
    c.ncol = (int64_t)K1 * K2; c.nbatch = 1;
    c.in_c = 1; c.in_i = (int64_t)K1 * K2;
    c.out_c = 1; c.out_i = (int64_t)K1 * K2;
    return run_pass<false>(p, c, t2, k, s);
}

// k (Kd) -> x (Nd): inverse passes, / prod(Kd), then x sn (apply_sn) or
// / sn (divide_sn).  k is not modified.
int pfft_inverse(nufft_plan_s* p, const float2* k, float2* x, bool apply_sn, bool divide_sn,
                 cudaStream_t s) {
    const int nd = p->ndim;
    const int N0 = p->Nd[0], N1 = p->Nd[1];
    const int K0 = p->Kd[0], K1 = p->Kd[1];
    const int last = nd - 1;
    const int NL = p->Nd[last], KL = p->Kd[last];
    float2* t1 = p->d_padin;
    if (nd == 2) {
        PfftPass b = base_pass(p, 0, true);
        b.n_in = K0; b.n_out = N0;
        b.ncol = K1; b.nbatch = 1;
        b.in_c = 1; b.in_i = K1;
        b.out_c = 1; b.out_i = K1;
        NUFFT_TRY(run_pass<false>(p, b, k, t1, s));
    } else {
        const int K2 = p->Kd[2];
        float2* t2 = p->d_slabout;
        PfftPass c = base_pass(p, 0, true);
        c.n_in = K0; c.n_out = N0;
        c.ncol = (int64_t)K1 * K2; c.nbatch = 1;
        c.in_c = 1; c.in_i = (int64_t)K1 * K2;
        c.out_c = 1; c.out_i = (int64_t)K1 * K2;
        NUFFT_TRY(run_pass<false>(p, c, k, t2, s));
        PfftPass b = base_pass(p, 1, true);
        b.n_in = K1; b.n_out = N1;
        b.ncol = K2; b.nbatch = N0;
        b.in_b = (int64_t)K1 * K2; b.in_c = 1; b.in_i = K2;
        b.out_b = (int64_t)N1 * K2; b.out_c = 1; b.out_i = K2;
        NUFFT_TRY(run_pass<false>(p, b, t2, t1, s));
    }
    PfftPass a = base_pass(p, last, true);
    a.n_in = KL;
    a.n_out = NL;
    a.ncol = (nd == 3) ? (int64_t)N0 * N1 : N0;
    a.nbatch = 1;
    a.in_c = KL; a.in_i = 1;
    a.out_c = NL; a.out_i = 1;
    a.norm = (float)(1.0 / (double)p->prodK);
    a.scale_out = divide_sn ? 2 : (apply_sn ? 1 : 0);
    a.sa = (nd == 3) ? sn_ptr(p, 0) : nullptr;
    a.sb = (nd == 3) ? sn_ptr(p, 1) : sn_ptr(p, 0);
    a.nb = (nd == 3) ? N1 : N0;
    a.sl = sn_ptr(p, last);
    return run_pass<true>(p, a, t1, x, s);
}

}  // namespace nufft

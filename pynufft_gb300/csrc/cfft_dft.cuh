// Small in-register DFTs for the coil-batched FFT passes (cfft.cu):
// V[q] = sum_r v[r] exp(-+2 pi i r q / R) for R in {2, 3, 4, 5, 6, 8, 10},
// the sign + for the inverse.  6 and 10 are prime-factor (Good-Thomas)
// compositions of 2 x 3 and 2 x 5, which need no twiddles: with
// n = (N2 n1 + N1 n2) mod N and k = CRT(k1 mod N1, k2 mod N2), exp(-2 pi i
// n k / N) = exp(-2 pi i n1 k1 / N1) exp(-2 pi i n2 k2 / N2).  Host and
// device, so the host tests can check them against the naive sums.
#pragma once
#include <cuda_runtime.h>

namespace nufft {
namespace cdft {

__host__ __device__ __forceinline__ float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 scl(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// -i a (forward) or +i a (inverse)
template <bool INV>
__host__ __device__ __forceinline__ float2 mi(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
__host__ __device__ __forceinline__ float2 mul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft2(float2& a, float2& b) {
    const float2 s = add(a, b), d = sub(a, b);
    a = s;
    b = d;
}

// X1 = a0 - (a1 + a2) / 2 -+ i (sqrt 3 / 2)(a1 - a2), X2 the conjugate pair
template <bool INV>
__host__ __device__ __forceinline__ void dft3(float2& a0, float2& a1, float2& a2) {
    constexpr float h = 0.86602540378443865f;   // sin(2 pi / 3)
    const float2 t = add(a1, a2), d = scl(sub(a1, a2), h);
    const float2 m = sub(a0, scl(t, 0.5f));
    a0 = add(a0, t);
    a1 = add(m, mi<INV>(d));
    a2 = sub(m, mi<INV>(d));
}

template <bool INV>
__host__ __device__ __forceinline__ void dft4(float2& a, float2& b, float2& c, float2& d) {
    const float2 s02 = add(a, c), d02 = sub(a, c), s13 = add(b, d), d13 = mi<INV>(sub(b, d));
    a = add(s02, s13);
    b = add(d02, d13);
    c = sub(s02, s13);
    d = sub(d02, d13);
}

// X1 = a0 + c1 t1 + c2 t2 -+ i (s1 u1 + s2 u2), X4 its pair;
// X2 = a0 + c2 t1 + c1 t2 -+ i (s2 u1 - s1 u2), X3 its pair;
// t1 = a1 + a4, t2 = a2 + a3, u1 = a1 - a4, u2 = a2 - a3, c_m = cos(2 pi m / 5),
// s_m = sin(2 pi m / 5)
template <bool INV>
__host__ __device__ __forceinline__ void dft5(float2& a0, float2& a1, float2& a2, float2& a3,
                                              float2& a4) {
    constexpr float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;
    constexpr float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;
    const float2 t1 = add(a1, a4), t2 = add(a2, a3), u1 = sub(a1, a4), u2 = sub(a2, a3);
    const float2 p1 = add(a0, add(scl(t1, c1), scl(t2, c2)));
    const float2 p2 = add(a0, add(scl(t1, c2), scl(t2, c1)));
    const float2 q1 = mi<INV>(add(scl(u1, s1), scl(u2, s2)));
    const float2 q2 = mi<INV>(sub(scl(u1, s2), scl(u2, s1)));
    a0 = add(a0, add(t1, t2));
    a1 = add(p1, q1);
    a4 = sub(p1, q1);
    a2 = add(p2, q2);
    a3 = sub(p2, q2);
}

// 8 = 2 x 4 (decimation in time): X[q] = E[q] + W8^q O[q], X[q + 4] = E[q] - W8^q O[q]
template <bool INV>
__host__ __device__ __forceinline__ void dft8(float2 (&v)[8]) {
    constexpr float r = 0.70710678118654752f;
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    // W8^1 = (1 -+ i) / sqrt 2, W8^2 = -+i, W8^3 = (-1 -+ i) / sqrt 2
    const float2 w1 = INV ? make_float2(r, r) : make_float2(r, -r);
    const float2 w3 = INV ? make_float2(-r, r) : make_float2(-r, -r);
    o1 = mul(o1, w1);
    o2 = mi<INV>(o2);
    o3 = mul(o3, w3);
    v[0] = add(e0, o0); v[4] = sub(e0, o0);
    v[1] = add(e1, o1); v[5] = sub(e1, o1);
    v[2] = add(e2, o2); v[6] = sub(e2, o2);
    v[3] = add(e3, o3); v[7] = sub(e3, o3);
}

// 6 = 2 x 3: n = (3 n1 + 2 n2) mod 6, k = (3 k1 + 4 k2) mod 6
template <bool INV>
__host__ __device__ __forceinline__ void dft6(float2 (&v)[6]) {
    float2 a0 = v[0], a1 = v[2], a2 = v[4];    // n1 = 0: n = 0, 2, 4
    float2 b0 = v[3], b1 = v[5], b2 = v[1];    // n1 = 1: n = 3, 5, 1
    dft3<INV>(a0, a1, a2);
    dft3<INV>(b0, b1, b2);
    v[0] = add(a0, b0); v[3] = sub(a0, b0);    // k2 = 0: k = 0, 3
    v[4] = add(a1, b1); v[1] = sub(a1, b1);    // k2 = 1: k = 4, 1
    v[2] = add(a2, b2); v[5] = sub(a2, b2);    // k2 = 2: k = 2, 5
}

// 10 = 2 x 5: n = (5 n1 + 2 n2) mod 10, k = (5 k1 + 6 k2) mod 10
template <bool INV>
__host__ __device__ __forceinline__ void dft10(float2 (&v)[10]) {
    float2 a0 = v[0], a1 = v[2], a2 = v[4], a3 = v[6], a4 = v[8];   // n1 = 0
    float2 b0 = v[5], b1 = v[7], b2 = v[9], b3 = v[1], b4 = v[3];   // n1 = 1
    dft5<INV>(a0, a1, a2, a3, a4);
    dft5<INV>(b0, b1, b2, b3, b4);
    v[0] = add(a0, b0); v[5] = sub(a0, b0);    // k2 = 0: k = 0, 5
    v[6] = add(a1, b1); v[1] = sub(a1, b1);    // k2 = 1: k = 6, 1
    v[2] = add(a2, b2); v[7] = sub(a2, b2);    // k2 = 2: k = 2, 7
    v[8] = add(a3, b3); v[3] = sub(a3, b3);    // k2 = 3: k = 8, 3
    v[4] = add(a4, b4); v[9] = sub(a4, b4);    // k2 = 4: k = 4, 9
}

template <int R, bool INV>
__host__ __device__ __forceinline__ void dft(float2 (&v)[R]) {
    if constexpr (R == 2) dft2<INV>(v[0], v[1]);
    else if constexpr (R == 3) dft3<INV>(v[0], v[1], v[2]);
    else if constexpr (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 5) dft5<INV>(v[0], v[1], v[2], v[3], v[4]);
    else if constexpr (R == 6) dft6<INV>(v);
    else if constexpr (R == 8) dft8<INV>(v);
    else if constexpr (R == 10) dft10<INV>(v);
    else static_assert(R == 2, "radix not built");
}

constexpr int kCW = 8;   // transforms (contiguous batch elements) per block of a pass

// Stockham stage of radix R after stages whose radices multiply to NS:
// butterfly j reads elements j + r L / R, scales element r by
// W_{NS R}^{r (j mod NS)}, and writes the R-point DFT to
// (j / NS) NS R + (j mod NS) + r NS.  After the last stage the L outputs are
// in natural order.
template <int L, int R, int NS>
struct Stage {
    static constexpr int NB = L / R;
    static_assert(L % (NS * R) == 0, "radices must divide the length");
    __host__ __device__ static int in_index(int j, int r) { return j + r * NB; }
    __host__ __device__ static int out_index(int j, int r) {
        return (j / NS) * NS * R + (j % NS) + r * NS;
    }
    __host__ __device__ static int tw_index(int j, int r) { return r * (j % NS) * (L / (NS * R)); }
};

template <int L, int R0, int R1, int R2>
struct Plan3 {
    static_assert(R0 * R1 * R2 == L, "three radices of L");
    using S0 = Stage<L, R0, 1>;
    using S1 = Stage<L, R1, R0>;
    using S2 = Stage<L, R2, R0 * R1>;
    static constexpr int T = (L / R0 > L / R1) ? ((L / R0 > L / R2) ? L / R0 : L / R2)
                                               : ((L / R1 > L / R2) ? L / R1 : L / R2);
    static constexpr int THREADS = kCW * T;
    // rows in shared memory, unpadded: the first stage's writes, rows R0
    // apart, share banks, but padding them (row l at l + l / R0) cost more
    // index arithmetic on every access than the conflicts (32-coil radial
    // pair 0.486 -> 0.480 ms, 8-coil kooshball 20.19 -> 19.99 ms unpadded)
    __host__ __device__ static int row(int l) { return l; }
    static constexpr int ROWS = L;
    static constexpr size_t SMEM = sizeof(float2) * ((size_t)ROWS * kCW + L);
};

}  // namespace cdft
}  // namespace nufft

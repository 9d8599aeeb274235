// Host emulation of one coil-batched FFT pass transform (cfft.cu): the same
// stage index arithmetic, twiddle indices and small DFTs (cfft_dft.cuh), run
// serially.  Reads "L lin lout inv" and lin complex inputs (re im per line)
// on stdin, writes lout complex outputs.  Built and driven by
// test_cfft_host.py, which compares with numpy.fft.
#include "../pynufft_gb300/csrc/cfft_dft.cuh"

#include <cmath>
#include <cstdio>
#include <vector>

using namespace nufft::cdft;

template <typename P, typename S, int R, bool INV>
static void stage(std::vector<float2>& buf, const std::vector<float2>& tw, const float2* in,
                  int lin, float2* out, int lout) {
    std::vector<float2> vals((size_t)S::NB * R);
    for (int j = 0; j < S::NB; ++j) {
        float2 v[R];
        for (int r = 0; r < R; ++r) {
            const int l = S::in_index(j, r);
            if (in) {
                v[r] = l < lin ? in[l] : make_float2(0.f, 0.f);
            } else {
                v[r] = buf[P::row(l)];
                if (r > 0) {
                    float2 t = tw[S::tw_index(j, r)];
                    if (INV) t.y = -t.y;
                    v[r] = mul(v[r], t);
                }
            }
        }
        dft<R, INV>(v);
        for (int r = 0; r < R; ++r) vals[(size_t)j * R + r] = v[r];
    }
    for (int j = 0; j < S::NB; ++j)
        for (int r = 0; r < R; ++r) {
            const int l = S::out_index(j, r);
            if (out) {
                if (l < lout) out[l] = vals[(size_t)j * R + r];
            } else {
                buf[P::row(l)] = vals[(size_t)j * R + r];
            }
        }
}

template <int L, int R0, int R1, int R2, bool INV>
static void run(const std::vector<float2>& x, int lin, int lout, std::vector<float2>& y) {
    using P = Plan3<L, R0, R1, R2>;
    std::vector<float2> tw(L), buf(P::ROWS);
    for (int m = 0; m < L; ++m) {
        const double a = -2.0 * M_PI * m / L;
        tw[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    stage<P, typename P::S0, R0, INV>(buf, tw, x.data(), lin, nullptr, 0);
    stage<P, typename P::S1, R1, INV>(buf, tw, nullptr, 0, nullptr, 0);
    stage<P, typename P::S2, R2, INV>(buf, tw, nullptr, 0, y.data(), lout);
}

template <bool INV>
static bool dispatch(int L, const std::vector<float2>& x, int lin, int lout, std::vector<float2>& y) {
    switch (L) {   // the radix plans of cfft.cu's run_len
        case 640: run<640, 10, 8, 8, INV>(x, lin, lout, y); return true;
        case 512: run<512, 8, 8, 8, INV>(x, lin, lout, y); return true;
        case 384: run<384, 6, 8, 8, INV>(x, lin, lout, y); return true;
        case 320: run<320, 5, 8, 8, INV>(x, lin, lout, y); return true;
        case 256: run<256, 4, 8, 8, INV>(x, lin, lout, y); return true;
        case 192: run<192, 6, 4, 8, INV>(x, lin, lout, y); return true;
        case 160: run<160, 5, 4, 8, INV>(x, lin, lout, y); return true;
        case 128: run<128, 2, 8, 8, INV>(x, lin, lout, y); return true;
        default: return false;
    }
}

int main() {
    int L, lin, lout, inv;
    if (std::scanf("%d %d %d %d", &L, &lin, &lout, &inv) != 4) return 2;
    std::vector<float2> x(lin), y(lout);
    for (int l = 0; l < lin; ++l) {
        double re, im;
        if (std::scanf("%lf %lf", &re, &im) != 2) return 2;
        x[l] = make_float2((float)re, (float)im);
    }
    const bool ok = inv ? dispatch<true>(L, x, lin, lout, y) : dispatch<false>(L, x, lin, lout, y);
    if (!ok) return 3;
    for (int l = 0; l < lout; ++l) std::printf("%.9e %.9e\n", y[l].x, y[l].y);
    return 0;
}

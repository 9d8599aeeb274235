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

__global__ void scale_kernel(ImgGeom g, const float2* __restrict__ in, float2* __restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.n_img;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = (e / g.B) % g.prodN;
        int n[3] = {0, 0, 0};
        for (int d = g.ndim - 1; d >= 0; --d) {
            n[d] = (int)(c % g.N[d]);
            c /= g.N[d];
        }
        const float s = sn_of(g, n);
        const float2 v = in[e];
        out[e] = make_float2(v.x * s, v.y * s);
    }
}

// grid[k] = x[k] * (sn[k] if apply_sn) * (-i (k_a - N_a/2) if dom_axis == a)
// for k inside the Nd corner, 0 elsewhere.
__global__ void pad_kernel(ImgGeom g, const float2* __restrict__ xx, float2* __restrict__ grid,
                           int apply_sn, int dom_axis) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.n_grid;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(e % g.B);
        int64_t c = e / g.B;
        const int64_t inst = c / g.prodK;
        c -= inst * g.prodK;
        int n[3] = {0, 0, 0};
        bool inside = true;
        int64_t ni = 0, stride = 1;
        for (int d = g.ndim - 1; d >= 0; --d) {
            n[d] = (int)(c % g.K[d]);
            c /= g.K[d];
            inside = inside && (n[d] < g.N[d]);
            ni += (int64_t)n[d] * stride;
            stride *= g.N[d];
        }
        float2 v = make_float2(0.f, 0.f);
        if (inside) {
            v = __ldg(xx + (inst * g.prodN + ni) * g.B + b);
            if (apply_sn) {
                const float s = sn_of(g, n);
                v.x *= s;
                v.y *= s;
            }
            if (dom_axis >= 0) {
                const float a = (float)n[dom_axis] - 0.5f * (float)g.N[dom_axis];
                v = make_float2(a * v.y, -a * v.x);
            }
        }
        grid[e] = v;
    }
}

// xx[n] = grid[n] / prod(Kd) * (sn[n] if apply_sn) / (sn[n] if divide_sn)
__global__ void crop_kernel(ImgGeom g, const float2* __restrict__ grid, float2* __restrict__ xx,
                            int apply_sn, int divide_sn, float norm) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < g.n_img;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(e % g.B);
        int64_t c = e / g.B;
        const int64_t inst = c / g.prodN;
        c -= inst * g.prodN;
        int n[3] = {0, 0, 0};
        int64_t ki = 0, stride = 1;
        for (int d = g.ndim - 1; d >= 0; --d) {
            n[d] = (int)(c % g.N[d]);
            c /= g.N[d];
            ki += (int64_t)n[d] * stride;
            stride *= g.K[d];
        }
        float2 v = __ldg(grid + (inst * g.prodK + ki) * g.B + b);
        float s = norm;
        if (apply_sn) s *= sn_of(g, n);
        v.x *= s;
        v.y *= s;
        if (divide_sn) {
            const float t = sn_of(g, n);
            v.x /= t;
            v.y /= t;
        }
        xx[e] = v;
    }
}

static int blocks_for(const nufft_plan_s* p, int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)p->num_sms * 32));
}

int launch_scale(const nufft_plan_s* p, const float2* in, float2* out, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    scale_kernel<<<blocks_for(p, g.n_img), 256, 0, s>>>(g, in, out);
    return check_launch("scale_kernel");
}

int launch_pad(const nufft_plan_s* p, const float2* xx, float2* grid, bool apply_sn,
               int dom_axis, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    pad_kernel<<<blocks_for(p, g.n_grid), 256, 0, s>>>(g, xx, grid, apply_sn ? 1 : 0, dom_axis);
    return check_launch("pad_kernel");
}

int launch_crop(const nufft_plan_s* p, const float2* grid, float2* xx, bool apply_sn,
                bool divide_sn, cudaStream_t s) {
    ImgGeom g = img_geom(p);
    const float norm = (float)(1.0 / (double)p->prodK);
    crop_kernel<<<blocks_for(p, g.n_img), 256, 0, s>>>(g, grid, xx, apply_sn ? 1 : 0,
                                                        divide_sn ? 1 : 0, norm);
    return check_launch("crop_kernel");
}

int fft_init(nufft_plan_s* p) {
    int n[3] = {p->Kd[0], p->Kd[1], p->Kd[2]};
    const int B = p->B;
    int istride, idist, batch;
    if (B == 1) {
        istride = 1;
        idist = (int)p->prodK;
        batch = p->ninst;
    } else {
        istride = B;
        idist = 1;
        batch = B;  // executed once per instance
    }
    NUFFT_CUFFT_TRY(cufftPlanMany(&p->fft, p->ndim, n, n, istride, idist, n, istride, idist,
                                  CUFFT_C2C, batch));
    p->fft_ok = true;
    return NUFFT_OK;
}

int fft_exec(nufft_plan_s* p, float2* grid, int direction, cudaStream_t s) {
    NUFFT_CUFFT_TRY(cufftSetStream(p->fft, s));
    const int dir = (direction < 0) ? CUFFT_FORWARD : CUFFT_INVERSE;
    if (p->B == 1 || p->ninst == 1) {
        NUFFT_CUFFT_TRY(cufftExecC2C(p->fft, reinterpret_cast<cufftComplex*>(grid),
                                     reinterpret_cast<cufftComplex*>(grid), dir));
    } else {
        for (int i = 0; i < p->ninst; ++i) {
            cufftComplex* g = reinterpret_cast<cufftComplex*>(grid + (size_t)i * p->prodK * p->B);
            NUFFT_CUFFT_TRY(cufftExecC2C(p->fft, g, g, dir));
        }
    }
    return NUFFT_OK;
}

}  // namespace nufft

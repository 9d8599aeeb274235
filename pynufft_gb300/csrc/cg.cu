// solve(y, 'cg', maxiter): conjugate gradients on the k-space normal operator.
//
// Reference semantics (linalg/solve_cpu.py:256-288): A = spH . sp as a
// LinearOperator over prod(Kd) unknowns, b = y2k(y), x0 = 0, and
// scipy.sparse.linalg.cg's recursion (rho = r^H r, alpha = rho / p^H A p,
// beta = rho_new / rho) with its stopping rule: stop at the top of an
// iteration when ||r|| < max(atol, rtol*||b||).  The k-space solution is
// mapped back with k2xx and divided by sn (solve_cpu.py:286-287).
//
// Every coil of every instance is an independent system with its own scalars.
// All scalars live on the device: the loop of maxiter iterations is captured
// once into a CUDA graph and replayed, with no host round trip per iteration.
// p^H A p is evaluated as ||sp p||^2 from the interpolated samples, which
// A = spH sp makes equal (the same quadratic form, one rounding apart).
// A system that has met its tolerance freezes (its kernels skip it), which
// reproduces the early return of scipy.  Vectors are complex64; the products
// inside dots and norms are float32 and are accumulated in FP64 (runs of 8
// elements in float32, then FP64), reduced in a fixed order so repeated
// solves give identical scalars.
#include "nufft_internal.cuh"

#include <algorithm>

namespace nufft {

struct CGSys {
    double rho, rho_prev, tol;
    double pq_re, pq_im, al_re, al_im;
    int done, iters, breakdown, maxiter;
    int xpend;   // x += alpha p of the last step not applied yet
};

struct CGGeom {
    int B, ninst, S;        // coils, instances, systems = ninst * B
    int64_t prodK;
    int nblk;               // reduction blocks per instance
    int Q;                  // threads per coil in a reduction block (power of 2)
};

// per-system partial sums of conj(a).b (complex) or |a|^2 (real, imag = 0)
template <bool NORM>
__device__ void block_dot(const CGGeom& g, const float2* __restrict__ a,
                          const float2* __restrict__ bvec, double2* __restrict__ part) {
    __shared__ double2 red[256];
    const int inst = blockIdx.y;
    const int t = threadIdx.x, b = t % g.B, q = t / g.B;
    const int64_t chunk = (g.prodK + g.nblk - 1) / g.nblk;
    const int64_t c0 = blockIdx.x * chunk, c1 = min(g.prodK, c0 + chunk);
    double sre = 0.0, sim = 0.0;
    int64_t c = c0 + q;
    while (c < c1) {
        float fre = 0.f, fim = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (c < c1) {
                const size_t e = ((size_t)inst * g.prodK + c) * g.B + b;
                const float2 va = a[e];
                if (NORM) {
                    fre = fmaf(va.x, va.x, fmaf(va.y, va.y, fre));
                } else {
                    const float2 vb = bvec[e];
                    fre = fmaf(va.x, vb.x, fmaf(va.y, vb.y, fre));
                    fim = fmaf(va.x, vb.y, fmaf(-va.y, vb.x, fim));
                }
            }
            c += g.Q;
        }
        sre += fre;
        sim += fim;
    }
    red[t] = make_double2(sre, sim);
    __syncthreads();
    for (int o = g.Q / 2; o > 0; o >>= 1) {
        if (q < o) {
            red[t].x += red[t + o * g.B].x;
            red[t].y += red[t + o * g.B].y;
        }
        __syncthreads();
    }
    if (q == 0) part[((size_t)inst * g.nblk + blockIdx.x) * g.B + b] = red[t];
}

// Sum of one system's per-block partials by a whole block (launched with one
// block of kSumThreads threads per system): strided partial sums, then a
// fixed-order tree, so the result does not depend on timing.  Every thread
// of the block receives the total.
constexpr int kSumThreads = 256;
__device__ double2 sum_parts(const CGGeom& g, const double2* part, int s) {
    __shared__ double2 red[kSumThreads];
    const int inst = s / g.B, b = s % g.B;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < g.nblk; k += blockDim.x) {
        const double2 v = part[((size_t)inst * g.nblk + k) * g.B + b];
        re += v.x;
        im += v.y;
    }
    red[threadIdx.x] = make_double2(re, im);
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            red[threadIdx.x].x += red[threadIdx.x + o].x;
            red[threadIdx.x].y += red[threadIdx.x + o].y;
        }
        __syncthreads();
    }
    return red[0];
}

// r = b (already in r), x = 0; rho = ||b||^2; tol = max(atol, rtol ||b||)
__global__ void cg_norm_kernel(CGGeom g, const float2* __restrict__ r, double2* __restrict__ part) {
    block_dot<true>(g, r, nullptr, part);
}

__global__ void cg_init_sys_kernel(CGGeom g, const double2* __restrict__ part,
                                   CGSys* __restrict__ sys, double rtol, double atol, int maxiter) {
    const int s = blockIdx.x;   // one block per system
    const double rho = sum_parts(g, part, s).x;
    if (threadIdx.x != 0) return;
    const double bn = sqrt(rho);
    CGSys st{};
    st.rho = rho;
    st.rho_prev = 1.0;
    st.tol = fmax(atol, rtol * bn);
    st.maxiter = maxiter;
    st.done = (bn == 0.0) || (bn < st.tol) || (maxiter <= 0) ? 1 : 0;
    sys[s] = st;
}

// x += alpha p for the previous step (deferred from cg_axpy_kernel, so that
// pass reads neither x nor p: the same operations on the same values, one
// pass later), then p = r (first iteration) or p = r + beta p; grid (nblk,
// ninst), thread t serves coil t % B like the reductions
__global__ void cg_update_p_kernel(CGGeom g, const CGSys* __restrict__ sys,
                                   const float2* __restrict__ r, float2* __restrict__ p,
                                   float2* __restrict__ x) {
    const int inst = blockIdx.y;
    const int t = threadIdx.x, b = t % g.B, q = t / g.B;
    const CGSys& st = sys[inst * g.B + b];
    const bool ux = st.xpend, up = !st.done;
    if (!ux && !up) return;
    const bool first = st.iters == 0;   // (nothing is pending then)
    const float beta = first ? 0.f : (float)(st.rho / st.rho_prev);
    const float ar = (float)st.al_re, ai = (float)st.al_im;
    const int64_t chunk = (g.prodK + g.nblk - 1) / g.nblk;
    const int64_t c0 = blockIdx.x * chunk, c1 = min(g.prodK, c0 + chunk);
    for (int64_t c = c0 + q; c < c1; c += g.Q) {
        const size_t e = ((size_t)inst * g.prodK + c) * g.B + b;
        if (ux) {
            const float2 pv = p[e];
            float2 xv = x[e];
            xv.x = fmaf(ar, pv.x, fmaf(-ai, pv.y, xv.x));
            xv.y = fmaf(ar, pv.y, fmaf(ai, pv.x, xv.y));
            x[e] = xv;
            if (up) {
                const float2 rv = r[e];
                p[e] = make_float2(fmaf(beta, pv.x, rv.x), fmaf(beta, pv.y, rv.y));
            }
        } else {
            const float2 rv = r[e];
            if (first) {
                p[e] = rv;
            } else {
                const float2 pv = p[e];
                p[e] = make_float2(fmaf(beta, pv.x, rv.x), fmaf(beta, pv.y, rv.y));
            }
        }
    }
}

// the step still pending after the last iteration: x += alpha p
__global__ void cg_xflush_kernel(CGGeom g, const CGSys* __restrict__ sys,
                                 const float2* __restrict__ p, float2* __restrict__ x) {
    const int inst = blockIdx.y;
    const int t = threadIdx.x, b = t % g.B, q = t / g.B;
    const CGSys& st = sys[inst * g.B + b];
    if (!st.xpend) return;
    const float ar = (float)st.al_re, ai = (float)st.al_im;
    const int64_t chunk = (g.prodK + g.nblk - 1) / g.nblk;
    const int64_t c0 = blockIdx.x * chunk, c1 = min(g.prodK, c0 + chunk);
    for (int64_t c = c0 + q; c < c1; c += g.Q) {
        const size_t e = ((size_t)inst * g.prodK + c) * g.B + b;
        const float2 pv = p[e];
        float2 xv = x[e];
        xv.x = fmaf(ar, pv.x, fmaf(-ai, pv.y, xv.x));
        xv.y = fmaf(ar, pv.y, fmaf(ai, pv.x, xv.y));
        x[e] = xv;
    }
}

// p^H q with q = A^H A p is ||A p||^2: per-system partial sums of |y|^2 over
// the system's samples y = A p (instance inst's points, coil b), which are
// M-sized instead of prod(Kd)-sized (2M points: 16 MB read against the
// 268 MB of p and q; same layout of partials as block_dot).
__global__ void cg_ynorm_kernel(CGGeom g, const float2* __restrict__ yv,
                                const int64_t* __restrict__ inst_start,
                                double2* __restrict__ part) {
    __shared__ double2 red[256];
    const int inst = blockIdx.y;
    const int t = threadIdx.x, b = t % g.B, q = t / g.B;
    const int64_t m0 = inst_start[inst], mi = inst_start[inst + 1] - m0;
    const int64_t chunk = (mi + g.nblk - 1) / g.nblk;
    const int64_t c0 = blockIdx.x * chunk, c1 = min(mi, c0 + chunk);
    double acc = 0.0;
    int64_t c = c0 + q;
    while (c < c1) {
        float f = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (c < c1) {
                const float2 v = yv[(size_t)(m0 + c) * g.B + b];
                f = fmaf(v.x, v.x, fmaf(v.y, v.y, f));
            }
            c += g.Q;
        }
        acc += f;
    }
    red[t] = make_double2(acc, 0.0);
    __syncthreads();
    for (int o = g.Q / 2; o > 0; o >>= 1) {
        if (q < o) red[t].x += red[t + o * g.B].x;
        __syncthreads();
    }
    if (q == 0) part[((size_t)inst * g.nblk + blockIdx.x) * g.B + b] = red[t];
}

__global__ void cg_alpha_kernel(CGGeom g, const double2* __restrict__ part, CGSys* __restrict__ sys) {
    const int s = blockIdx.x;   // one block per system
    if (sys[s].done) {
        // this iteration's cg_update_p_kernel has applied its pending step
        if (threadIdx.x == 0) sys[s].xpend = 0;
        return;
    }
    const double2 pq = sum_parts(g, part, s);
    if (threadIdx.x != 0) return;
    CGSys st = sys[s];
    st.pq_re = pq.x;
    st.pq_im = pq.y;
    const double den = pq.x * pq.x + pq.y * pq.y;
    if (!(pq.x > 0.0) || !isfinite(den) || den == 0.0) {
        st.breakdown = 1;
        st.done = 1;
        st.al_re = st.al_im = 0.0;
        st.xpend = 0;
    } else {
        // alpha = rho / pq (complex); x += alpha p follows in the next update
        st.al_re = st.rho * pq.x / den;
        st.al_im = -st.rho * pq.y / den;
        st.xpend = 1;
    }
    sys[s] = st;
}

// r -= alpha q; partial ||r||^2 (x += alpha p waits for the next
// cg_update_p_kernel, which reads p anyway)
__global__ void cg_axpy_kernel(CGGeom g, const CGSys* __restrict__ sys, const float2* __restrict__ q,
                               float2* __restrict__ r, double2* __restrict__ part) {
    __shared__ double2 red[256];
    const int inst = blockIdx.y;
    const int t = threadIdx.x, b = t % g.B, qq = t / g.B;
    const CGSys& st = sys[inst * g.B + b];
    const bool active = !st.done;
    const float ar = (float)st.al_re, ai = (float)st.al_im;
    const int64_t chunk = (g.prodK + g.nblk - 1) / g.nblk;
    const int64_t c0 = blockIdx.x * chunk, c1 = min(g.prodK, c0 + chunk);
    double acc = 0.0;
    int64_t c = c0 + qq;
    while (c < c1) {
        float f = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (c < c1) {
                const size_t e = ((size_t)inst * g.prodK + c) * g.B + b;
                float2 rv = r[e];
                if (active) {
                    const float2 qv = q[e];
                    rv.x = fmaf(-ar, qv.x, fmaf(ai, qv.y, rv.x));
                    rv.y = fmaf(-ar, qv.y, fmaf(-ai, qv.x, rv.y));
                    r[e] = rv;
                }
                f = fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, f));
            }
            c += g.Q;
        }
        acc += f;
    }
    red[t] = make_double2(acc, 0.0);
    __syncthreads();
    for (int o = g.Q / 2; o > 0; o >>= 1) {
        if (qq < o) red[t].x += red[t + o * g.B].x;
        __syncthreads();
    }
    if (qq == 0) part[((size_t)inst * g.nblk + blockIdx.x) * g.B + b] = red[t];
}

__global__ void cg_finalize_kernel(CGGeom g, const double2* __restrict__ part, CGSys* __restrict__ sys) {
    const int s = blockIdx.x;   // one block per system
    if (sys[s].done) return;
    const double rho = sum_parts(g, part, s).x;
    if (threadIdx.x != 0) return;
    CGSys st = sys[s];
    st.rho_prev = st.rho;
    st.rho = rho;
    st.iters += 1;
    if (sqrt(st.rho) < st.tol || st.iters >= st.maxiter) st.done = 1;
    sys[s] = st;
}

// iterations per captured graph; solves needing more relaunch it and check
// convergence on the host between launches
static const int kChunk = 32;

void free_cg(nufft_plan_s* p) {
    if (p->cg_init_exec) cudaGraphExecDestroy(p->cg_init_exec);
    if (p->cg_iter_exec) cudaGraphExecDestroy(p->cg_iter_exec);
    p->cg_init_exec = p->cg_iter_exec = nullptr;
    p->cg_y = nullptr;
    cudaFree(p->d_cg); p->d_cg = nullptr;
    cudaFree(p->d_cgs); p->d_cgs = nullptr;
    cudaFree(p->d_part); p->d_part = nullptr;
}

static CGGeom cg_geom(const nufft_plan_s* p) {
    CGGeom g{};
    g.B = p->B;
    g.ninst = p->ninst;
    g.S = p->B * p->ninst;
    g.prodK = p->prodK;
    int Q = 1;
    while (Q * 2 * p->B <= 256) Q *= 2;
    g.Q = Q;
    // enough blocks for 8 per SM in total (latency hiding for the streaming
    // vector kernels); their partials are summed by a whole block per system
    int64_t want = std::max<int64_t>(1, (int64_t)p->num_sms * 8 / std::max(1, p->ninst));
    g.nblk = (int)std::min<int64_t>(want, std::max<int64_t>(1, p->prodK / (8 * Q)));
    return g;
}

// Initial residual: x = 0, r = b = y2k(y), per-system scalars.
static int issue_init(nufft_plan_s* p, const CGGeom& g, const float2* y, int maxiter, double rtol,
                      double atol, cudaStream_t s) {
    const int64_t n = (int64_t)p->ninst * p->prodK * p->B;
    float2* xk = p->d_cg;
    float2* r = xk + n;
    CGSys* sys = reinterpret_cast<CGSys*>(p->d_cgs);
    double2* part = reinterpret_cast<double2*>(p->d_part);
    const dim3 rgrid(g.nblk, g.ninst);
    NUFFT_CUDA_TRY(cudaMemsetAsync(xk, 0, sizeof(float2) * n, s));
    NUFFT_TRY(launch_y2k_grid(p, y, r, s));
    cg_norm_kernel<<<rgrid, g.B * g.Q, 0, s>>>(g, r, part);
    NUFFT_TRY(check_launch("cg_norm_kernel"));
    cg_init_sys_kernel<<<g.S, kSumThreads, 0, s>>>(g, part, sys, rtol, atol, maxiter);
    return check_launch("cg_init_sys_kernel");
}

// `iters` CG iterations; systems that are done (converged or at maxiter) skip.
static int issue_iters(nufft_plan_s* p, const CGGeom& g, int iters, cudaStream_t s) {
    const int64_t n = (int64_t)p->ninst * p->prodK * p->B;
    float2* xk = p->d_cg;
    float2* r = xk + n;
    float2* pv = r + n;
    float2* q = pv + n;
    CGSys* sys = reinterpret_cast<CGSys*>(p->d_cgs);
    double2* part = reinterpret_cast<double2*>(p->d_part);
    const dim3 rgrid(g.nblk, g.ninst);
    const int rthreads = g.B * g.Q;
    for (int it = 0; it < iters; ++it) {
        cg_update_p_kernel<<<rgrid, rthreads, 0, s>>>(g, sys, r, pv, xk);
        NUFFT_TRY(check_launch("cg_update_p_kernel"));
        NUFFT_TRY(launch_k2y(p, pv, p->d_ybuf, s));          // q = spH sp p
        cg_ynorm_kernel<<<rgrid, rthreads, 0, s>>>(g, p->d_ybuf, p->d_inst_start, part);
        NUFFT_TRY(check_launch("cg_ynorm_kernel"));           // p^H q = ||sp p||^2
        NUFFT_TRY(launch_y2k_grid(p, p->d_ybuf, q, s));
        cg_alpha_kernel<<<g.S, kSumThreads, 0, s>>>(g, part, sys);
        NUFFT_TRY(check_launch("cg_alpha_kernel"));
        cg_axpy_kernel<<<rgrid, rthreads, 0, s>>>(g, sys, q, r, part);
        NUFFT_TRY(check_launch("cg_axpy_kernel"));
        cg_finalize_kernel<<<g.S, kSumThreads, 0, s>>>(g, part, sys);
        NUFFT_TRY(check_launch("cg_finalize_kernel"));
    }
    return NUFFT_OK;
}

template <typename F>
static int capture(cudaGraphExec_t* exec, F&& body) {
    static thread_local cudaStream_t cap = nullptr;
    if (!cap) NUFFT_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    if (*exec) { cudaGraphExecDestroy(*exec); *exec = nullptr; }
    cudaGraph_t graph = nullptr;
    NUFFT_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    int st = body(cap);
    cudaError_t ce = cudaStreamEndCapture(cap, &graph);
    if (st != NUFFT_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (ce != cudaSuccess) {
        set_error(std::string("nufft_solve_cg: capture failed: ") + cudaGetErrorString(ce));
        return NUFFT_ECUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        *exec = nullptr;
        set_error(std::string("nufft_solve_cg: instantiate: ") + cudaGetErrorString(ie));
        return NUFFT_ECUDA;
    }
    return NUFFT_OK;
}

int solve_cg(nufft_plan_s* p, const float2* y, float2* x, int maxiter, double rtol, double atol,
             int* iters_out, cudaStream_t s) {
    if (p->B > 256) {
        set_error("nufft_solve_cg: batch > 256 is not supported");
        return NUFFT_EUNSUPPORTED;
    }
    const int64_t n = (int64_t)p->ninst * p->prodK * p->B;
    if (maxiter < 0) maxiter = (int)std::min<int64_t>(10 * p->prodK, 0x7fffffff);  // scipy's default
    CGGeom g = cg_geom(p);
    if (!p->d_cg) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_cg, sizeof(float2) * 4 * n));
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_cgs, sizeof(CGSys) * g.S));
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_part, sizeof(double2) * (size_t)g.nblk * g.ninst * g.B));
        p->dev_bytes += sizeof(float2) * 4 * n + sizeof(CGSys) * g.S +
                        sizeof(double2) * (size_t)g.nblk * g.ninst * g.B;
    }
    const int chunk = std::max(1, std::min(maxiter, kChunk));
    if (!p->cg_init_exec || p->cg_y != (const void*)y || p->cg_maxiter != maxiter ||
        p->cg_rtol != rtol || p->cg_atol != atol || !p->cg_iter_exec || p->cg_chunk != chunk) {
        // one uncaptured gridding pass first: it creates any lazily allocated
        // buffers and sets kernel attributes outside the capture
        NUFFT_TRY(launch_y2k_grid(p, p->d_ybuf, p->d_grid, s));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
        NUFFT_TRY(capture(&p->cg_init_exec, [&](cudaStream_t cs) {
            return issue_init(p, g, y, maxiter, rtol, atol, cs);
        }));
        NUFFT_TRY(capture(&p->cg_iter_exec, [&](cudaStream_t cs) {
            return issue_iters(p, g, chunk, cs);
        }));
        p->cg_y = y;
        p->cg_maxiter = maxiter;
        p->cg_rtol = rtol;
        p->cg_atol = atol;
        p->cg_chunk = chunk;
    }
    NUFFT_CUDA_TRY(cudaGraphLaunch(p->cg_init_exec, s));
    std::vector<CGSys> hs(g.S);
    for (int done_it = 0; done_it < maxiter; done_it += chunk) {
        NUFFT_CUDA_TRY(cudaGraphLaunch(p->cg_iter_exec, s));
        if (done_it + chunk >= maxiter) break;
        // more than one chunk: stop launching once every system is done
        NUFFT_CUDA_TRY(cudaMemcpyAsync(hs.data(), p->d_cgs, sizeof(CGSys) * g.S,
                                       cudaMemcpyDeviceToHost, s));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
        bool all = true;
        for (const CGSys& st : hs) all = all && st.done;
        if (all) break;
    }

    // the last step, then the k-space solution -> image: k2xx, divide by sn
    float2* xk = p->d_cg;
    {
        const dim3 rgrid(g.nblk, g.ninst);
        cg_xflush_kernel<<<rgrid, g.B * g.Q, 0, s>>>(g, reinterpret_cast<const CGSys*>(p->d_cgs),
                                                     xk + 2 * n, xk);
        NUFFT_TRY(check_launch("cg_xflush_kernel"));
    }
    NUFFT_TRY(image_from_spectrum(p, xk, x, false, true, s));

    if (iters_out) {
        NUFFT_CUDA_TRY(cudaMemcpyAsync(hs.data(), p->d_cgs, sizeof(CGSys) * g.S,
                                       cudaMemcpyDeviceToHost, s));
        NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
        int mx = 0, brk = 0;
        for (const CGSys& st : hs) { mx = std::max(mx, st.iters); brk |= st.breakdown; }
        *iters_out = mx;
        if (brk) {
            set_error("nufft_solve_cg: breakdown (p^H A p not positive or not finite)");
            return NUFFT_ECG_BREAKDOWN;
        }
    }
    return NUFFT_OK;
}

}  // namespace nufft

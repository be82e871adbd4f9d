// Batched real 2D FFTs over z-planes (FP64), replacing the FFTW r2c/c2r plane
// transforms of fftw3_dns_module.f90:72-130 that the reference calls once per
// z-plane and per field (33*nz plane transforms per step).
//
// Transform definition (FFTW plan dims (ny, nx), row-major, x fastest):
//   r2c: F[ky][kx] = sum_{y,x} f[y][x] e^{-2 pi i (kx x/nx + ky y/ny)},
//        kx = 0..nx/2, unnormalised (fftw3_dns_module.f90:106).
//   c2r: inverse c2c along y for every kx column, then a 1D c2r of length nx
//        along each row that uses Re only of the kx=0 and kx=nx/2 entries,
//        then /(nx*ny) (fftw3_dns_module.f90:127-130).  This fixes the result
//        for non-Hermitian input (derivatives at the Nyquist wavenumbers).
//
// Algorithm: Stockham autosort passes (radix 4, 2, 3) in shared memory.  The
// y pass loads a block of CX kx-columns of one plane (coalesced rows of CX
// complex values); the x pass loads RX rows of one plane and runs the length-nx
// real transform as a length-nx/2 complex transform plus a pack/unpack step.
// Twiddles come from tables built on the host in long double.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "dns3d_internal.cuh"

namespace dns3d {

bool fft_length_supported(int n) {
    if (n < 2) return false;
    int m = n;
    while (m % 2 == 0) m /= 2;
    if (m % 3 == 0) m /= 3;
    return m == 1;
}

FftPlan1D make_plan(int n) {
    FftPlan1D p{};
    p.n = n;
    int m = n;
    int s = 0;
    while (m % 4 == 0 && s < kMaxStages) { p.radix[s++] = 4; m /= 4; }
    while (m % 2 == 0 && s < kMaxStages) { p.radix[s++] = 2; m /= 2; }
    while (m % 3 == 0 && s < kMaxStages) { p.radix[s++] = 3; m /= 3; }
    p.nstages = s;
    return p;
}

namespace {

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }

// One Stockham pass over `count` transforms of length n stored at a[c*ld + t].
// SIGN = -1 forward (e^{-i}), +1 inverse.  tw[t] = e^{-2 pi i t/n}.
template <int SIGN, typename C>
__device__ void stockham_pass(const C* __restrict__ a, C* __restrict__ b, int count,
                              int ld, int n, int R, int Ns, const C* __restrict__ tw) {
    using R_t = decltype(C::x);
    const int nb = n / R;
    const int total = count * nb;
    const int tstep = n / (Ns * R);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int c = t / nb;
        const int j = t - c * nb;
        const int k = j % Ns;
        const C* src = a + c * ld;
        C v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < R) v[r] = src[j + r * nb];
        if (k != 0) {
#pragma unroll
            for (int r = 1; r < 4; ++r) {
                if (r < R) {
                    C w = tw[r * k * tstep];
                    if (SIGN > 0) w.y = -w.y;
                    v[r] = cmul(v[r], w);
                }
            }
        }
        C y[4];
        if (R == 4) {
            const C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
            const C s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
            // (SIGN i) * d13
            const C id13 = SIGN > 0 ? mk<C>(-d13.y, d13.x) : mk<C>(d13.y, -d13.x);
            y[0] = cadd(s02, s13);
            y[2] = csub(s02, s13);
            y[1] = cadd(d02, id13);
            y[3] = csub(d02, id13);
        } else if (R == 2) {
            y[0] = cadd(v[0], v[1]);
            y[1] = csub(v[0], v[1]);
        } else {  // R == 3
            const R_t h = (R_t)0.86602540378443864676;  // sqrt(3)/2
            const C t1 = cadd(v[1], v[2]);
            const C d = csub(v[1], v[2]);
            const C m = mk<C>(v[0].x - (R_t)0.5 * t1.x, v[0].y - (R_t)0.5 * t1.y);
            // (SIGN i h) * d
            const C id = SIGN > 0 ? mk<C>(-h * d.y, h * d.x) : mk<C>(h * d.y, -h * d.x);
            y[0] = cadd(v[0], t1);
            y[1] = cadd(m, id);
            y[2] = csub(m, id);
        }
        C* dst = b + c * ld;
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < R) dst[base + q * Ns] = y[q];
    }
}

// Runs all passes; returns the buffer holding the result.
template <int SIGN, typename C>
__device__ C* stockham(C* a, C* b, int count, int ld, const FftPlan1D& pl, const C* __restrict__ tw) {
    int Ns = 1;
    for (int s = 0; s < pl.nstages; ++s) {
        const int R = pl.radix[s];
        stockham_pass<SIGN>(a, b, count, ld, pl.n, R, Ns, tw);
        __syncthreads();
        C* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Complex FFT along y of kx-columns [kx0, kx0+cx) of one plane.
// grid (ceil(nxhp/cx), nplanes, nf); smem 2*cx*(ny+1) double2.
template <int SIGN, typename C>
__global__ void __launch_bounds__(256) k_fft_y(FieldsT<C> src, FieldsT<C> dst, GridDev g, FftPlan1D pl,
                                               const C* __restrict__ tw, int cx, int ncols_total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* smem = reinterpret_cast<C*>(smem_raw);
    const int ld = g.ny + 1;
    C* a = smem;
    C* b = smem + cx * ld;
    const int kx0 = blockIdx.x * cx;
    const size_t plane = (size_t)blockIdx.y * g.nm;
    const C* __restrict__ s = src.p[blockIdx.z] + plane;
    C* d = dst.p[blockIdx.z] + plane;
    const int ncol = min(cx, ncols_total - kx0);
    for (int t = threadIdx.x; t < g.ny * cx; t += blockDim.x) {
        const int y = t / cx, c = t - y * cx;
        if (c < ncol) a[c * ld + y] = s[(size_t)y * g.nxhp + kx0 + c];
    }
    __syncthreads();
    C* r = stockham<SIGN>(a, b, ncol, ld, pl, tw);
    for (int t = threadIdx.x; t < g.ny * cx; t += blockDim.x) {
        const int y = t / cx, c = t - y * cx;
        if (c < ncol) d[(size_t)y * g.nxhp + kx0 + c] = r[c * ld + y];
    }
}

// c2r along x for rows [row0, row0+rx) (row = plane*ny + y) of one field.
// grid (ceil(nrows/rx), nf); smem 2*rx*(nx/2+2) double2.
template <typename T>
__global__ void __launch_bounds__(256) k_c2r_x(FieldsT<typename Cx<T>::type> src, FieldsT<T> dst, GridDev g,
                                               FftPlan1D pl, const typename Cx<T>::type* __restrict__ tw_nx2,
                                               const typename Cx<T>::type* __restrict__ tw_nx, int rx,
                                               int nrows) {
    using C = typename Cx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* smem = reinterpret_cast<C*>(smem_raw);
    const int n2 = g.nxh;
    const int ld = n2 + 2;
    C* a = smem;
    C* b = smem + rx * ld;
    const int row0 = blockIdx.x * rx;
    const int nr = min(rx, nrows - row0);
    const C* __restrict__ s = src.p[blockIdx.y] + (size_t)row0 * g.nxhp;
    C* d = reinterpret_cast<C*>(dst.p[blockIdx.y] + (size_t)row0 * g.nx);
    for (int t = threadIdx.x; t < nr * g.nxhp; t += blockDim.x) {
        const int r = t / g.nxhp, k = t - r * g.nxhp;
        C v = s[t];
        if (k == 0 || k == n2) v.y = (T)0;  // c2r uses Re only at kx = 0, nx/2
        a[r * ld + k] = v;
    }
    __syncthreads();
    // Z[k] = (X[k] + conj(X[n2-k])) + i e^{+2 pi i k/nx} (X[k] - conj(X[n2-k]))
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        const C xa = a[r * ld + k];
        const C xb = a[r * ld + n2 - k];
        const C sm = mk<C>(xa.x + xb.x, xa.y - xb.y);
        const C df = mk<C>(xa.x - xb.x, xa.y + xb.y);
        C w = tw_nx[k];
        w.y = -w.y;
        const C p = cmul(w, df);
        b[r * ld + k] = mk<C>(sm.x - p.y, sm.y + p.x);
    }
    __syncthreads();
    C* res = stockham<+1>(b, a, nr, ld, pl, tw_nx2);
    const T sc = (T)g.inv_nxny;
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        const C z = res[r * ld + k];
        d[(size_t)r * n2 + k] = mk<C>(z.x * sc, z.y * sc);
    }
}

// r2c along x: rows of nx reals -> nxhp complex.
template <typename T>
__global__ void __launch_bounds__(256) k_r2c_x(FieldsT<T> src, FieldsT<typename Cx<T>::type> dst, GridDev g,
                                               FftPlan1D pl, const typename Cx<T>::type* __restrict__ tw_nx2,
                                               const typename Cx<T>::type* __restrict__ tw_nx, int rx,
                                               int nrows) {
    using C = typename Cx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* smem = reinterpret_cast<C*>(smem_raw);
    const int n2 = g.nxh;
    const int ld = n2 + 2;
    C* a = smem;
    C* b = smem + rx * ld;
    const int row0 = blockIdx.x * rx;
    const int nr = min(rx, nrows - row0);
    const C* __restrict__ s = reinterpret_cast<const C*>(src.p[blockIdx.y] + (size_t)row0 * g.nx);
    C* d = dst.p[blockIdx.y] + (size_t)row0 * g.nxhp;
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        a[r * ld + k] = s[t];  // z[m] = x[2m] + i x[2m+1]
    }
    __syncthreads();
    C* res = stockham<-1>(a, b, nr, ld, pl, tw_nx2);
    C* out = (res == a) ? b : a;
    // X[k] = E + e^{-2 pi i k/nx} O,  E = (Z[k]+conj(Z[n2-k]))/2,  O = (Z[k]-conj(Z[n2-k]))/(2i)
    for (int t = threadIdx.x; t < nr * (n2 + 1); t += blockDim.x) {
        const int r = t / (n2 + 1), k = t - r * (n2 + 1);
        const C za = res[r * ld + (k == n2 ? 0 : k)];
        const C zb = res[r * ld + (k == 0 ? 0 : n2 - k)];
        const T hf = (T)0.5;
        const C e = mk<C>(hf * (za.x + zb.x), hf * (za.y - zb.y));
        const C o = mk<C>(hf * (za.y + zb.y), -hf * (za.x - zb.x));
        const C p = cmul(tw_nx[k], o);
        out[r * ld + k] = mk<C>(e.x + p.x, e.y + p.y);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nr * g.nxhp; t += blockDim.x) {
        const int r = t / g.nxhp, k = t - r * g.nxhp;
        d[(size_t)r * g.nxhp + k] = out[r * ld + k];
    }
}

int pick_cx(int ny) {
    int cx = 2048 / ny;
    if (cx > 16) cx = 16;
    if (cx < 1) cx = 1;
    return cx;
}
int pick_rx(int n2) {
    int rx = 2048 / n2;
    if (rx > 16) rx = 16;
    if (rx < 1) rx = 1;
    return rx;
}

template <typename C>
C* upload_table(int n, int count) {
    // e^{-2 pi i t/n}, t < count, computed in long double and rounded once.
    std::vector<C> h(count);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int t = 0; t < count; ++t) {
        const long double ang = -2.0L * pi * (long double)t / (long double)n;
        h[t].x = (decltype(C::x))cosl(ang);
        h[t].y = (decltype(C::x))sinl(ang);
    }
    C* d = nullptr;
    if (cudaMalloc(&d, sizeof(C) * count) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(C) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

// Raised to the device's opt-in maximum: the limit belongs to the kernel
// function and is shared by every handle (every grid) in the process.
template <typename K>
cudaError_t smem_attr(K k, int bytes) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev))) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k))) return e;
    const int limit = optin - (int)fa.sharedSizeBytes;  // static + dynamic <= opt-in maximum
    if (bytes > limit) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
}

// round(2^62 e^{-2 pi i t/n}), t < count, from the long double values.
longlong2* upload_table_q62(int n, int count) {
    std::vector<longlong2> h(count);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int t = 0; t < count; ++t) {
        const long double ang = -2.0L * pi * (long double)t / (long double)n;
        h[t].x = llroundl(ldexpl(cosl(ang), 62));
        h[t].y = llroundl(ldexpl(sinl(ang), 62));
    }
    longlong2* d = nullptr;
    if (cudaMalloc(&d, sizeof(longlong2) * count) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(longlong2) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

}  // namespace

cudaError_t fft_setup(FftCtx& ctx, const GridDev& g) {
    ctx.py = make_plan(g.ny);
    ctx.px2 = make_plan(g.nxh);
    ctx.use_ct = fft_ct_supported(g.ny, g.nxh);
    ctx.tw_ny = upload_table<double2>(g.ny, g.ny);
    ctx.tw_nx2 = upload_table<double2>(g.nxh, g.nxh);
    ctx.tw_nx = upload_table<double2>(g.nx, g.nxh + 1);
    ctx.tw32_ny = upload_table<float2>(g.ny, g.ny);
    ctx.tw32_nx2 = upload_table<float2>(g.nxh, g.nxh);
    ctx.tw32_nx = upload_table<float2>(g.nx, g.nxh + 1);
    if (!ctx.tw_ny || !ctx.tw_nx2 || !ctx.tw_nx || !ctx.tw32_ny || !ctx.tw32_nx2 || !ctx.tw32_nx)
        return cudaErrorMemoryAllocation;
    const char* f64 = std::getenv("DNS3D_FFT_FP64");
    ctx.fx = ctx.use_ct && !(f64 && f64[0] == '1');
    if (ctx.fx) {
        ctx.twq_ny = upload_table_q62(g.ny, g.ny);
        ctx.twq_nx2 = upload_table_q62(g.nxh, g.nxh);
        ctx.twq_nx = upload_table_q62(g.nx, g.nxh + 1);
        if (!ctx.twq_ny || !ctx.twq_nx2 || !ctx.twq_nx) return cudaErrorMemoryAllocation;
    }
    const int cx = pick_cx(g.ny);
    const int rx = pick_rx(g.nxh);
    const int sy = 2 * cx * (g.ny + 1) * (int)sizeof(double2);
    const int sx = 2 * rx * (g.nxh + 2) * (int)sizeof(double2);
    cudaError_t e;
    if ((e = smem_attr(k_fft_y<-1, double2>, sy)) || (e = smem_attr(k_fft_y<+1, double2>, sy)) ||
        (e = smem_attr(k_c2r_x<double>, sx)) || (e = smem_attr(k_r2c_x<double>, sx)) ||
        (e = smem_attr(k_fft_y<-1, float2>, sy / 2)) || (e = smem_attr(k_fft_y<+1, float2>, sy / 2)) ||
        (e = smem_attr(k_c2r_x<float>, sx / 2)) || (e = smem_attr(k_r2c_x<float>, sx / 2)))
        return e;
    return cudaSuccess;
}

void fft_release(FftCtx& ctx) {
    cudaFree(ctx.tw_ny);
    cudaFree(ctx.tw_nx2);
    cudaFree(ctx.tw_nx);
    cudaFree(ctx.tw32_ny);
    cudaFree(ctx.tw32_nx2);
    cudaFree(ctx.tw32_nx);
    cudaFree(ctx.twq_ny);
    cudaFree(ctx.twq_nx2);
    cudaFree(ctx.twq_nx);
    ctx.twq_ny = ctx.twq_nx2 = ctx.twq_nx = nullptr;
    ctx.tw_ny = ctx.tw_nx2 = ctx.tw_nx = nullptr;
    ctx.tw32_ny = ctx.tw32_nx2 = ctx.tw32_nx = nullptr;
}

namespace {

template <typename T>
cudaError_t c2r_impl(const FftCtx& ctx, const GridDev& g, FieldsT<typename Cx<T>::type> spec, FieldsT<T> phys,
                     FieldsT<typename Cx<T>::type> tmp, int nf, int nplanes, cudaStream_t s,
                     const typename Cx<T>::type* twy, const typename Cx<T>::type* twx2,
                     const typename Cx<T>::type* twx) {
    using C = typename Cx<T>::type;
    const int nrows = nplanes * g.ny;
    if constexpr (sizeof(T) == 8) {
        if (ctx.fx) {
            cudaError_t e = fft_fx_y<+1>(spec, tmp, g, nplanes, g.nxhp, nf, ctx.twq_ny, s);
            if (e) return e;
            if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_y_inverse");
            e = fft_fx_c2r_x(tmp, phys, RFields{}, g, nrows, nf, ctx.twq_nx2, ctx.twq_nx, s);
            if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_x_c2r");
            return e;
        }
    }
    if (ctx.use_ct) {
        cudaError_t e = fft_ct_y<+1, C>(spec, tmp, g, nplanes, g.nxhp, nf, twy, s);
        if (e) return e;
        if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_y_inverse" : "fft32_y_inverse");
        e = fft_ct_c2r_x<T>(tmp, phys, g, nrows, nf, twx2, twx, s);
        if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_x_c2r" : "fft32_x_c2r");
        return e;
    }
    const int cx = pick_cx(g.ny);
    dim3 gy((g.nxhp + cx - 1) / cx, nplanes, nf);
    k_fft_y<+1, C><<<gy, 256, 2 * cx * (g.ny + 1) * sizeof(C), s>>>(spec, tmp, g, ctx.py, twy, cx, g.nxhp);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_y_inverse" : "fft32_y_inverse");
    const int rx = pick_rx(g.nxh);
    dim3 gx((nrows + rx - 1) / rx, nf);
    k_c2r_x<T><<<gx, 256, 2 * rx * (g.nxh + 2) * sizeof(C), s>>>(tmp, phys, g, ctx.px2, twx2, twx, rx, nrows);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_x_c2r" : "fft32_x_c2r");
    return cudaGetLastError();
}

template <typename T>
cudaError_t r2c_impl(const FftCtx& ctx, const GridDev& g, FieldsT<T> phys, FieldsT<typename Cx<T>::type> spec,
                     int nf, int nplanes, cudaStream_t s, const typename Cx<T>::type* twy,
                     const typename Cx<T>::type* twx2, const typename Cx<T>::type* twx, int ncol,
                     bool host_src = false) {
    using C = typename Cx<T>::type;
    const int nrows = nplanes * g.ny;
    if (ncol <= 0 || ncol > g.nxhp) ncol = g.nxhp;
    if constexpr (sizeof(T) == 8) {
        if (ctx.fx) {
            cudaError_t e = fft_fx_r2c_x(phys, spec, g, nrows, nf, ctx.twq_nx2, ctx.twq_nx, host_src, s);
            if (e) return e;
            if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_x_r2c");
            e = fft_fx_y<-1>(spec, spec, g, nplanes, ncol, nf, ctx.twq_ny, s);
            if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_y_forward");
            return e;
        }
    }
    if (ctx.use_ct) {
        cudaError_t e = fft_ct_r2c_x<T>(phys, spec, g, nrows, nf, twx2, twx, s);
        if (e) return e;
        if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_x_r2c" : "fft32_x_r2c");
        e = fft_ct_y<-1, C>(spec, spec, g, nplanes, ncol, nf, twy, s);
        if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_y_forward" : "fft32_y_forward");
        return e;
    }
    const int rx = pick_rx(g.nxh);
    dim3 gx((nrows + rx - 1) / rx, nf);
    k_r2c_x<T><<<gx, 256, 2 * rx * (g.nxh + 2) * sizeof(C), s>>>(phys, spec, g, ctx.px2, twx2, twx, rx, nrows);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_x_r2c" : "fft32_x_r2c");
    const int cx = pick_cx(g.ny);
    dim3 gy((ncol + cx - 1) / cx, nplanes, nf);
    k_fft_y<-1, C><<<gy, 256, 2 * cx * (g.ny + 1) * sizeof(C), s>>>(spec, spec, g, ctx.py, twy, cx, ncol);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, sizeof(T) == 8 ? "fft_y_forward" : "fft32_y_forward");
    return cudaGetLastError();
}

}  // namespace

cudaError_t fft_c2r(const FftCtx& ctx, const GridDev& g, Fields spec, RFields phys, int nf, int nplanes,
                    cudaStream_t s, int slot0) {
    if (slot0 < 0 || slot0 + nf > ctx.tmp_fields || nf > kMaxFields) return cudaErrorInvalidValue;
    Fields tmp{};
    for (int f = 0; f < nf; ++f) tmp.p[f] = ctx.tmp + (size_t)(slot0 + f) * g.nm * g.nz;
    return c2r_impl<double>(ctx, g, spec, phys, tmp, nf, nplanes, s, ctx.tw_ny, ctx.tw_nx2, ctx.tw_nx);
}

cudaError_t fft_c2r_copy(const FftCtx& ctx, const GridDev& g, Fields spec, RFields phys, RFields copy, int nf,
                         int nplanes, cudaStream_t s) {
    if (!ctx.fx) return cudaErrorNotSupported;
    if (nf > ctx.tmp_fields || nf > kMaxFields) return cudaErrorInvalidValue;
    Fields tmp{};
    for (int f = 0; f < nf; ++f) tmp.p[f] = ctx.tmp + (size_t)f * g.nm * g.nz;
    cudaError_t e = fft_fx_y<+1>(spec, tmp, g, nplanes, g.nxhp, nf, ctx.twq_ny, s);
    if (e) return e;
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_y_inverse");
    e = fft_fx_c2r_x(tmp, phys, copy, g, nplanes * g.ny, nf, ctx.twq_nx2, ctx.twq_nx, s);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_x_c2r");
    return e;
}

cudaError_t fft_r2c(const FftCtx& ctx, const GridDev& g, RFields phys, Fields spec, int nf, int nplanes,
                    cudaStream_t s, int ncol, bool host_src) {
    if (nf > kMaxFields) return cudaErrorInvalidValue;
    return r2c_impl<double>(ctx, g, phys, spec, nf, nplanes, s, ctx.tw_ny, ctx.tw_nx2, ctx.tw_nx, ncol, host_src);
}

cudaError_t fft_c2r32(const FftCtx& ctx, const GridDev& g, FFields spec, FRFields phys, int nf, int nplanes,
                      cudaStream_t s) {
    if (nf > ctx.tmp_fields || nf > kMaxFields || !ctx.tmp32) return cudaErrorInvalidValue;
    FFields tmp{};
    for (int f = 0; f < nf; ++f) tmp.p[f] = ctx.tmp32 + (size_t)f * g.nm * g.nz;
    return c2r_impl<float>(ctx, g, spec, phys, tmp, nf, nplanes, s, ctx.tw32_ny, ctx.tw32_nx2, ctx.tw32_nx);
}

cudaError_t fft_r2c32(const FftCtx& ctx, const GridDev& g, FRFields phys, FFields spec, int nf, int nplanes,
                      cudaStream_t s, int ncol) {
    if (nf > kMaxFields) return cudaErrorInvalidValue;
    return r2c_impl<float>(ctx, g, phys, spec, nf, nplanes, s, ctx.tw32_ny, ctx.tw32_nx2, ctx.tw32_nx, ncol);
}

}  // namespace dns3d

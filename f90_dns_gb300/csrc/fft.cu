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

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// One Stockham pass over `count` transforms of length n stored at a[c*ld + t].
// SIGN = -1 forward (e^{-i}), +1 inverse.  tw[t] = e^{-2 pi i t/n}.
template <int SIGN>
__device__ void stockham_pass(const double2* __restrict__ a, double2* __restrict__ b, int count,
                              int ld, int n, int R, int Ns, const double2* __restrict__ tw) {
    const int nb = n / R;
    const int total = count * nb;
    const int tstep = n / (Ns * R);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int c = t / nb;
        const int j = t - c * nb;
        const int k = j % Ns;
        const double2* src = a + c * ld;
        double2 v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < R) v[r] = src[j + r * nb];
        if (k != 0) {
#pragma unroll
            for (int r = 1; r < 4; ++r) {
                if (r < R) {
                    double2 w = __ldg(&tw[r * k * tstep]);
                    if (SIGN > 0) w.y = -w.y;
                    v[r] = cmul(v[r], w);
                }
            }
        }
        double2 y[4];
        if (R == 4) {
            const double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
            const double2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
            // (SIGN i) * d13
            const double2 id13 = SIGN > 0 ? make_double2(-d13.y, d13.x) : make_double2(d13.y, -d13.x);
            y[0] = cadd(s02, s13);
            y[2] = csub(s02, s13);
            y[1] = cadd(d02, id13);
            y[3] = csub(d02, id13);
        } else if (R == 2) {
            y[0] = cadd(v[0], v[1]);
            y[1] = csub(v[0], v[1]);
        } else {  // R == 3
            const double h = 0.86602540378443864676;  // sqrt(3)/2
            const double2 t1 = cadd(v[1], v[2]);
            const double2 d = csub(v[1], v[2]);
            const double2 m = make_double2(v[0].x - 0.5 * t1.x, v[0].y - 0.5 * t1.y);
            // (SIGN i h) * d
            const double2 id = SIGN > 0 ? make_double2(-h * d.y, h * d.x) : make_double2(h * d.y, -h * d.x);
            y[0] = cadd(v[0], t1);
            y[1] = cadd(m, id);
            y[2] = csub(m, id);
        }
        double2* dst = b + c * ld;
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < R) dst[base + q * Ns] = y[q];
    }
}

// Runs all passes; returns the buffer holding the result.
template <int SIGN>
__device__ double2* stockham(double2* a, double2* b, int count, int ld, const FftPlan1D& pl,
                             const double2* __restrict__ tw) {
    int Ns = 1;
    for (int s = 0; s < pl.nstages; ++s) {
        const int R = pl.radix[s];
        stockham_pass<SIGN>(a, b, count, ld, pl.n, R, Ns, tw);
        __syncthreads();
        double2* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Complex FFT along y of kx-columns [kx0, kx0+cx) of one plane.
// grid (ceil(nxhp/cx), nplanes, nf); smem 2*cx*(ny+1) double2.
template <int SIGN>
__global__ void __launch_bounds__(256) k_fft_y(Fields src, Fields dst, GridDev g, FftPlan1D pl,
                                               const double2* __restrict__ tw, int cx) {
    extern __shared__ double2 smem[];
    const int ld = g.ny + 1;
    double2* a = smem;
    double2* b = smem + cx * ld;
    const int kx0 = blockIdx.x * cx;
    const size_t plane = (size_t)blockIdx.y * g.nm;
    const double2* __restrict__ s = src.p[blockIdx.z] + plane;
    double2* d = dst.p[blockIdx.z] + plane;
    const int ncol = min(cx, g.nxhp - kx0);
    for (int t = threadIdx.x; t < g.ny * cx; t += blockDim.x) {
        const int y = t / cx, c = t - y * cx;
        if (c < ncol) a[c * ld + y] = s[(size_t)y * g.nxhp + kx0 + c];
    }
    __syncthreads();
    double2* r = stockham<SIGN>(a, b, ncol, ld, pl, tw);
    for (int t = threadIdx.x; t < g.ny * cx; t += blockDim.x) {
        const int y = t / cx, c = t - y * cx;
        if (c < ncol) d[(size_t)y * g.nxhp + kx0 + c] = r[c * ld + y];
    }
}

// c2r along x for rows [row0, row0+rx) (row = plane*ny + y) of one field.
// grid (ceil(nrows/rx), nf); smem 2*rx*(nx/2+2) double2.
__global__ void __launch_bounds__(256) k_c2r_x(Fields src, RFields dst, GridDev g, FftPlan1D pl,
                                               const double2* __restrict__ tw_nx2,
                                               const double2* __restrict__ tw_nx, int rx,
                                               int nrows) {
    extern __shared__ double2 smem[];
    const int n2 = g.nxh;
    const int ld = n2 + 2;
    double2* a = smem;
    double2* b = smem + rx * ld;
    const int row0 = blockIdx.x * rx;
    const int nr = min(rx, nrows - row0);
    const double2* __restrict__ s = src.p[blockIdx.y] + (size_t)row0 * g.nxhp;
    double2* d = reinterpret_cast<double2*>(dst.p[blockIdx.y] + (size_t)row0 * g.nx);
    for (int t = threadIdx.x; t < nr * g.nxhp; t += blockDim.x) {
        const int r = t / g.nxhp, k = t - r * g.nxhp;
        double2 v = s[t];
        if (k == 0 || k == n2) v.y = 0.0;  // c2r uses Re only at kx = 0, nx/2
        a[r * ld + k] = v;
    }
    __syncthreads();
    // Z[k] = (X[k] + conj(X[n2-k])) + i e^{+2 pi i k/nx} (X[k] - conj(X[n2-k]))
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        const double2 xa = a[r * ld + k];
        const double2 xb = a[r * ld + n2 - k];
        const double2 sm = make_double2(xa.x + xb.x, xa.y - xb.y);
        const double2 df = make_double2(xa.x - xb.x, xa.y + xb.y);
        double2 w = __ldg(&tw_nx[k]);
        w.y = -w.y;
        const double2 p = cmul(w, df);
        b[r * ld + k] = make_double2(sm.x - p.y, sm.y + p.x);
    }
    __syncthreads();
    double2* res = stockham<+1>(b, a, nr, ld, pl, tw_nx2);
    const double sc = g.inv_nxny;
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        const double2 z = res[r * ld + k];
        d[(size_t)r * n2 + k] = make_double2(z.x * sc, z.y * sc);
    }
}

// r2c along x: rows of nx reals -> nxhp complex.
__global__ void __launch_bounds__(256) k_r2c_x(RFields src, Fields dst, GridDev g, FftPlan1D pl,
                                               const double2* __restrict__ tw_nx2,
                                               const double2* __restrict__ tw_nx, int rx,
                                               int nrows) {
    extern __shared__ double2 smem[];
    const int n2 = g.nxh;
    const int ld = n2 + 2;
    double2* a = smem;
    double2* b = smem + rx * ld;
    const int row0 = blockIdx.x * rx;
    const int nr = min(rx, nrows - row0);
    const double2* __restrict__ s =
        reinterpret_cast<const double2*>(src.p[blockIdx.y] + (size_t)row0 * g.nx);
    double2* d = dst.p[blockIdx.y] + (size_t)row0 * g.nxhp;
    for (int t = threadIdx.x; t < nr * n2; t += blockDim.x) {
        const int r = t / n2, k = t - r * n2;
        a[r * ld + k] = s[t];  // z[m] = x[2m] + i x[2m+1]
    }
    __syncthreads();
    double2* res = stockham<-1>(a, b, nr, ld, pl, tw_nx2);
    double2* out = (res == a) ? b : a;
    // X[k] = E + e^{-2 pi i k/nx} O,  E = (Z[k]+conj(Z[n2-k]))/2,  O = (Z[k]-conj(Z[n2-k]))/(2i)
    for (int t = threadIdx.x; t < nr * (n2 + 1); t += blockDim.x) {
        const int r = t / (n2 + 1), k = t - r * (n2 + 1);
        const double2 za = res[r * ld + (k == n2 ? 0 : k)];
        const double2 zb = res[r * ld + (k == 0 ? 0 : n2 - k)];
        const double2 e = make_double2(0.5 * (za.x + zb.x), 0.5 * (za.y - zb.y));
        const double2 o = make_double2(0.5 * (za.y + zb.y), -0.5 * (za.x - zb.x));
        const double2 p = cmul(__ldg(&tw_nx[k]), o);
        out[r * ld + k] = make_double2(e.x + p.x, e.y + p.y);
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

double2* upload_table(int n, int count) {
    // e^{-2 pi i t/n}, t < count, computed in long double and rounded once.
    std::vector<double2> h(count);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int t = 0; t < count; ++t) {
        const long double ang = -2.0L * pi * (long double)t / (long double)n;
        h[t] = make_double2((double)cosl(ang), (double)sinl(ang));
    }
    double2* d = nullptr;
    if (cudaMalloc(&d, sizeof(double2) * count) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(double2) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

}  // namespace

cudaError_t fft_setup(FftCtx& ctx, const GridDev& g) {
    ctx.py = make_plan(g.ny);
    ctx.px2 = make_plan(g.nxh);
    ctx.tw_ny = upload_table(g.ny, g.ny);
    ctx.tw_nx2 = upload_table(g.nxh, g.nxh);
    ctx.tw_nx = upload_table(g.nx, g.nxh + 1);
    if (!ctx.tw_ny || !ctx.tw_nx2 || !ctx.tw_nx) return cudaErrorMemoryAllocation;
    const int cx = pick_cx(g.ny);
    const int rx = pick_rx(g.nxh);
    const int sy = 2 * cx * (g.ny + 1) * (int)sizeof(double2);
    const int sx = 2 * rx * (g.nxh + 2) * (int)sizeof(double2);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_fft_y<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sy))) return e;
    if ((e = cudaFuncSetAttribute(k_fft_y<+1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sy))) return e;
    if ((e = cudaFuncSetAttribute(k_c2r_x, cudaFuncAttributeMaxDynamicSharedMemorySize, sx))) return e;
    if ((e = cudaFuncSetAttribute(k_r2c_x, cudaFuncAttributeMaxDynamicSharedMemorySize, sx))) return e;
    return cudaSuccess;
}

void fft_release(FftCtx& ctx) {
    cudaFree(ctx.tw_ny);
    cudaFree(ctx.tw_nx2);
    cudaFree(ctx.tw_nx);
    ctx.tw_ny = ctx.tw_nx2 = ctx.tw_nx = nullptr;
}

cudaError_t fft_c2r(const FftCtx& ctx, const GridDev& g, Fields spec, RFields phys, int nf,
                    int nplanes, cudaStream_t s) {
    if (nf > ctx.tmp_fields || nf > kMaxFields) return cudaErrorInvalidValue;
    Fields tmp{};
    for (int f = 0; f < nf; ++f) tmp.p[f] = ctx.tmp + (size_t)f * g.nm * g.nz;
    const int cx = pick_cx(g.ny);
    dim3 gy((g.nxhp + cx - 1) / cx, nplanes, nf);
    k_fft_y<+1><<<gy, 256, 2 * cx * (g.ny + 1) * sizeof(double2), s>>>(spec, tmp, g, ctx.py,
                                                                       ctx.tw_ny, cx);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_y_inverse");
    const int rx = pick_rx(g.nxh);
    const int nrows = nplanes * g.ny;
    dim3 gx((nrows + rx - 1) / rx, nf);
    k_c2r_x<<<gx, 256, 2 * rx * (g.nxh + 2) * sizeof(double2), s>>>(tmp, phys, g, ctx.px2,
                                                                    ctx.tw_nx2, ctx.tw_nx, rx, nrows);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_x_c2r");
    return cudaGetLastError();
}

cudaError_t fft_r2c(const FftCtx& ctx, const GridDev& g, RFields phys, Fields spec, int nf,
                    int nplanes, cudaStream_t s) {
    if (nf > kMaxFields) return cudaErrorInvalidValue;
    const int rx = pick_rx(g.nxh);
    const int nrows = nplanes * g.ny;
    dim3 gx((nrows + rx - 1) / rx, nf);
    k_r2c_x<<<gx, 256, 2 * rx * (g.nxh + 2) * sizeof(double2), s>>>(phys, spec, g, ctx.px2,
                                                                    ctx.tw_nx2, ctx.tw_nx, rx, nrows);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_x_r2c");
    const int cx = pick_cx(g.ny);
    dim3 gy((g.nxhp + cx - 1) / cx, nplanes, nf);
    k_fft_y<-1><<<gy, 256, 2 * cx * (g.ny + 1) * sizeof(double2), s>>>(spec, spec, g, ctx.py,
                                                                       ctx.tw_ny, cx);
    if (ctx.hook) ctx.hook(ctx.hook_ctx, "fft_y_forward");
    return cudaGetLastError();
}

}  // namespace dns3d

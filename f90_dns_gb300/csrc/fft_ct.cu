// Plane transforms with the transform length fixed at compile time: the same
// transforms as fft.cu (FFTW's r2c / non-Hermitian c2r conventions), for the
// lengths that the supported grids use, with
//  - the radix schedule, the per-pass index arithmetic and the loop trip
//    counts resolved by the compiler (no runtime division in the passes);
//  - radix-8 butterflies in registers (a length-128 transform is 3 passes
//    instead of 4, length 512 is 3 instead of 5);
//  - one shared-memory buffer per CTA: each pass reads all of a thread's
//    butterfly inputs into registers, synchronises, and writes the outputs
//    in place, so a CTA holds ~2048 complex values in 16-33 KB (no opt-in);
//  - the y pass over a flattened (plane, kx) column index, so grids whose
//    nx/2+1 columns do not fill a CTA waste no lanes.
// Lengths outside the instantiated set use the generic kernels of fft.cu.
#include <type_traits>

#include "cvt.cuh"
#include "dns3d_internal.cuh"
#include "ragged.cuh"
#include "tc.cuh"

namespace dns3d {

// Instantiated lengths: ny in {16..512}, nx/2 in {16..256}, 2^a 3^b.
#define DNS3D_CT_Y_LENGTHS(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512)
#define DNS3D_CT_X_LENGTHS(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256)

namespace {

constexpr int kThreads = 256;

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// (SIGN i) a
template <int SIGN, typename C> __device__ __forceinline__ C mul_si(C a) {
    return SIGN > 0 ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x);
}

// ------------------------------------------------------------------ 64-bit fixed point
// The FP64 path's transforms run in block fixed point on the integer pipes:
// this GPU issues FP64 arithmetic at 1/64 of its FP32 rate, and the FP64
// plane transforms were bound by it.  One transform (a y column or an x row)
// is scaled by the power of two that gives its largest input component
// B <= 53 significant bits (as an FP64 mantissa has), with B small enough
// that no partial DFT can leave int64 (a length-N DFT grows a modulus at most
// N-fold); butterflies then add exactly, and every twiddle product is formed
// exactly in 128 bits and rounded once to the transform's grid.  Twiddles and
// constants are Q62 integers (value * 2^62).  The result differs from an FP64
// transform's by the same order as that transform's own rounding error
// (normwise ~2^-B per rounding step).
using fx2 = longlong2;

__device__ __forceinline__ long long fx_round62(__int128 v) {
    return (long long)((v + ((__int128)1 << 61)) >> 62);
}
// x c for a Q62 constant c
__device__ __forceinline__ long long fx_mulq(long long x, long long c) { return fx_round62((__int128)x * c); }

template <> __device__ __forceinline__ fx2 cmul<fx2>(fx2 a, fx2 w) {
    const __int128 re = (__int128)a.x * w.x - (__int128)a.y * w.y;
    const __int128 im = (__int128)a.x * w.y + (__int128)a.y * w.x;
    return mk<fx2>(fx_round62(re), fx_round62(im));
}

constexpr long long kFxInvSqrt2 = 3260954456333195553LL;  // round(2^62 / sqrt 2)
constexpr long long kFxSqrt3h = 3993837246235628775LL;    // round(2^62 sqrt(3) / 2)

template <typename C> __host__ __device__ constexpr bool is_fx() { return std::is_same<C, fx2>::value; }

// Register DFTs, natural-order output, w = e^{SIGN 2 pi i / R}.
template <int SIGN, typename C> __device__ __forceinline__ void dft2(C* v) {
    const C a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft4(C* v) {
    const C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const C s13 = cadd(v[1], v[3]), d13 = mul_si<SIGN>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}

// y[q] = E[q] + w8^q O[q], y[q+4] = E[q] - w8^q O[q] (E, O: 4-point DFTs of
// the even and odd inputs); w8 = (1 + SIGN i)/sqrt2, w8^2 = SIGN i,
// w8^3 = (-1 + SIGN i)/sqrt2.
template <int SIGN, typename C> __device__ __forceinline__ void dft8(C* v) {
    using R = decltype(C::x);
    C e[4] = {v[0], v[2], v[4], v[6]};
    C o[4] = {v[1], v[3], v[5], v[7]};
    dft4<SIGN>(e);
    dft4<SIGN>(o);
    C t1, t3;
    if constexpr (is_fx<C>()) {
        const long long s = SIGN;
        t1 = mk<C>(fx_mulq(o[1].x - s * o[1].y, kFxInvSqrt2), fx_mulq(o[1].y + s * o[1].x, kFxInvSqrt2));
        t3 = mk<C>(fx_mulq(-o[3].x - s * o[3].y, kFxInvSqrt2), fx_mulq(-o[3].y + s * o[3].x, kFxInvSqrt2));
    } else {
        const R h = (R)0.70710678118654752440;
        const R s = (R)SIGN;
        t1 = mk<C>(h * (o[1].x - s * o[1].y), h * (o[1].y + s * o[1].x));
        t3 = mk<C>(h * (-o[3].x - s * o[3].y), h * (-o[3].y + s * o[3].x));
    }
    const C t2 = mul_si<SIGN>(o[2]);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft3(C* v) {
    using R = decltype(C::x);
    const C t1 = cadd(v[1], v[2]);
    const C d = csub(v[1], v[2]);
    C m, id;
    if constexpr (is_fx<C>()) {
        // t/2 rounded half up; sqrt(3)/2 as a Q62 constant
        m = mk<C>(v[0].x - ((t1.x + 1) >> 1), v[0].y - ((t1.y + 1) >> 1));
        const long long hx = fx_mulq(d.x, kFxSqrt3h), hy = fx_mulq(d.y, kFxSqrt3h);
        id = SIGN > 0 ? mk<C>(-hy, hx) : mk<C>(hy, -hx);
    } else {
        const R h = (R)0.86602540378443864676;  // sqrt(3)/2
        m = mk<C>(v[0].x - (R)0.5 * t1.x, v[0].y - (R)0.5 * t1.y);
        id = SIGN > 0 ? mk<C>(-h * d.y, h * d.x) : mk<C>(h * d.y, -h * d.x);
    }
    v[0] = cadd(v[0], t1);
    v[1] = cadd(m, id);
    v[2] = csub(m, id);
}

template <int R, int SIGN, typename C> __device__ __forceinline__ void dft(C* v) {
    if constexpr (R == 8) dft8<SIGN>(v);
    else if constexpr (R == 4) dft4<SIGN>(v);
    else if constexpr (R == 2) dft2<SIGN>(v);
    else dft3<SIGN>(v);
}

// field pointer i of a by-value FieldsT without a dynamic index into the
// parameter block (which would copy the array to local memory)
template <typename P> __device__ __forceinline__ P* field_ptr(const FieldsT<P>& f, int i) {
    P* r = f.p[0];
#pragma unroll
    for (int k = 1; k < kMaxFields; ++k)
        if (i == k) r = f.p[k];
    return r;
}

__host__ __device__ constexpr int next_radix(int m) { return m % 8 == 0 ? 8 : (m % 4 == 0 ? 4 : (m % 2 == 0 ? 2 : 3)); }

// Transforms per CTA: a power of two near 2048 / N, in [1, 64].
__host__ __device__ constexpr int per_cta(int n) {
    int c = 1;
    while (c * 2 * n <= 2048 && c < 64) c *= 2;
    return c;
}

// Shared-memory slot of element t of one transform.  FP32 passes insert one
// padding slot after every 16 elements, so that a Stockham pass's writes at
// stride R (8 for the radix-8 passes) fall in distinct banks instead of in
// two: those passes are bound by shared-memory throughput.  The FP64 and
// fixed-point passes (16-byte elements, bound by their arithmetic) keep the
// plain layout, which needs fewer registers.
template <typename C> __host__ __device__ constexpr int sw(int t) {
    return std::is_same<C, float2>::value ? t + (t >> 4) : t;
}
// Slots per transform: elements 0..N (slot sw(N) holds an x pass's kx = nx/2 input).
template <typename C> __host__ __device__ constexpr int ld_of(int n) { return sw<C>(n) + 1; }

// One Stockham pass (radix R, Ns finished sub-length) over CNT transforms of
// length N stored at buf[c*LD + sw(t)], in place: all inputs of the thread's
// butterflies are read into registers before a barrier, then written.
// tw[t] = e^{-2 pi i t / N}.
template <int N, int R, int NS, int SIGN, int CNT, int LD, typename C>
__device__ __forceinline__ void ct_pass(C* buf, const C* __restrict__ tw) {
    constexpr int NB = N / R;
    constexpr int TSTEP = N / (NS * R);
    constexpr int TOTAL = CNT * NB;
    constexpr int PER = (TOTAL + kThreads - 1) / kThreads;
    C v[PER][R];
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int t = threadIdx.x + p * kThreads;
        if (TOTAL % kThreads == 0 || t < TOTAL) {
            const int c = t / NB, j = t - c * NB;
            const C* src = buf + c * LD;
#pragma unroll
            for (int r = 0; r < R; ++r) v[p][r] = src[sw<C>(j + r * NB)];
            if constexpr (NS > 1) {
                const int k = j % NS;
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    C w = __ldg(&tw[r * k * TSTEP]);
                    if (SIGN > 0) w.y = -w.y;
                    v[p][r] = cmul(v[p][r], w);
                }
            }
            dft<R, SIGN>(v[p]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int t = threadIdx.x + p * kThreads;
        if (TOTAL % kThreads == 0 || t < TOTAL) {
            const int c = t / NB, j = t - c * NB;
            const int k = j % NS;
            C* dst = buf + c * LD;
            const int o = (j / NS) * NS * R + k;
#pragma unroll
            for (int q = 0; q < R; ++q) dst[sw<C>(o + q * NS)] = v[p][q];
        }
    }
    __syncthreads();
}

template <int N, int NS, int SIGN, int CNT, int LD, typename C>
__device__ __forceinline__ void ct_fft(C* buf, const C* __restrict__ tw) {
    if constexpr (NS < N) {
        constexpr int R = next_radix(N / NS);
        ct_pass<N, R, NS, SIGN, CNT, LD>(buf, tw);
        ct_fft<N, NS * R, SIGN, CNT, LD>(buf, tw);
    }
}

// y pass: complex transforms of length N = ny along the (plane, kx) columns
// with kx < ncol (ncol = nx/2+1, or fewer when the 2/3 filter discards the
// rest); CX columns per CTA taken from the flattened index plane * ncol + kx.
// grid (ceil(nplanes * ncol / CX), 1, nf).
// Block bx of field f; buf holds at least ct_buf_elems(N) values.
template <int N, int SIGN, typename C>
__device__ __forceinline__ void fft_y_body(const FieldsT<C>& src, const FieldsT<C>& dst, const GridDev& g,
                                           int nplanes, int ncol, const C* __restrict__ tw, int bx, int f,
                                           C* buf) {
    constexpr int CX = per_cta(N);
    constexpr int LD = ld_of<C>(N);
    const long long ncols = (long long)nplanes * ncol;
    const long long vc = (long long)bx * CX + (threadIdx.x % CX);
    const bool live = vc < ncols;
    size_t base = 0;
    if (live) {
        const int p = (int)(vc / ncol);
        const int kx = (int)(vc - (long long)p * ncol);
        base = (size_t)p * g.nm + kx;
    }
    const C* __restrict__ s = field_ptr(src, f);
    C* d = field_ptr(dst, f);
    constexpr int ROWS_PER_ITER = kThreads / CX;  // CX divides kThreads
    constexpr int ITERS = N / ROWS_PER_ITER;
    static_assert(N % ROWS_PER_ITER == 0, "rows split evenly over the threads");
    const int c = threadIdx.x % CX, y0 = threadIdx.x / CX;
    // all of a thread's loads are issued before any is used
    C v[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it)
        v[it] = live ? s[base + (size_t)(y0 + it * ROWS_PER_ITER) * g.nxhp] : mk<C>(0, 0);
#pragma unroll
    for (int it = 0; it < ITERS; ++it) buf[c * LD + sw<C>(y0 + it * ROWS_PER_ITER)] = v[it];
    __syncthreads();
    ct_fft<N, 1, SIGN, CX, LD>(buf, tw);
    if (live) {
#pragma unroll
        for (int it = 0; it < ITERS; ++it)
            d[base + (size_t)(y0 + it * ROWS_PER_ITER) * g.nxhp] = buf[c * LD + sw<C>(y0 + it * ROWS_PER_ITER)];
    }
}

template <int N, int SIGN, typename C>
__global__ void __launch_bounds__(kThreads) k_fft_y_ct(FieldsT<C> src, FieldsT<C> dst, GridDev g, int nplanes,
                                                       int ncol, const C* __restrict__ tw) {
    __shared__ C buf[per_cta(N) * ld_of<C>(N)];
    fft_y_body<N, SIGN, C>(src, dst, g, nplanes, ncol, tw, blockIdx.x, blockIdx.z, buf);
}

// c2r along x, N = nx/2: RX rows per CTA (row = plane * ny + y).  Packs the
// nx/2+1 inputs of a row (Re only at kx = 0, nx/2) into Z[k] =
// (X[k] + conj(X[N-k])) + i e^{+2 pi i k/nx} (X[k] - conj(X[N-k])), runs the
// inverse length-N transform and writes z[m] = (x[2m], x[2m+1]) / (nx ny).
template <int N, typename T>
__device__ __forceinline__ void c2r_x_body(const FieldsT<typename Cx<T>::type>& src, const FieldsT<T>& dst,
                                           const GridDev& g, int nrows,
                                           const typename Cx<T>::type* __restrict__ tw_n,
                                           const typename Cx<T>::type* __restrict__ tw_nx, int bx, int f,
                                           typename Cx<T>::type* buf) {
    using C = typename Cx<T>::type;
    constexpr int RX = per_cta(N);
    constexpr int LD = ld_of<C>(N);
    const int row0 = bx * RX;
    const C* __restrict__ s = field_ptr(src, f);
    C* d = reinterpret_cast<C*>(field_ptr(dst, f));
    const int nxhp = N + 1;
    constexpr int ITERS = RX * N / kThreads;
    static_assert((RX * N) % kThreads == 0, "rows split evenly over the threads");
    // all of a thread's loads are issued before any is used
    C xa[ITERS], xb[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        xa[it] = xb[it] = mk<C>(0, 0);
        if (row0 + r < nrows) {
            const C* row = s + (size_t)(row0 + r) * nxhp;
            xa[it] = row[k];
            xb[it] = row[N - k];
        }
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        C a = xa[it], b = xb[it];
        if (k == 0) {
            a.y = 0;
            b.y = 0;
        }
        const C sm = mk<C>(a.x + b.x, a.y - b.y);
        const C df = mk<C>(a.x - b.x, a.y + b.y);
        C w = __ldg(&tw_nx[k]);
        w.y = -w.y;
        const C p = cmul(w, df);
        buf[r * LD + sw<C>(k)] = mk<C>(sm.x - p.y, sm.y + p.x);
    }
    __syncthreads();
    ct_fft<N, 1, +1, RX, LD>(buf, tw_n);
    const T sc = (T)g.inv_nxny;
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        if (row0 + r < nrows) {
            const C z = buf[r * LD + sw<C>(k)];
            d[(size_t)(row0 + r) * N + k] = mk<C>(z.x * sc, z.y * sc);
        }
    }
}

template <int N, typename T>
__global__ void __launch_bounds__(kThreads) k_c2r_x_ct(FieldsT<typename Cx<T>::type> src, FieldsT<T> dst,
                                                       GridDev g, int nrows,
                                                       const typename Cx<T>::type* __restrict__ tw_n,
                                                       const typename Cx<T>::type* __restrict__ tw_nx) {
    __shared__ typename Cx<T>::type buf[per_cta(N) * ld_of<typename Cx<T>::type>(N)];
    c2r_x_body<N, T>(src, dst, g, nrows, tw_n, tw_nx, blockIdx.x, blockIdx.y, buf);
}

// r2c along x, N = nx/2: z[m] = x[2m] + i x[2m+1], forward length-N
// transform, X[k] = E + e^{-2 pi i k/nx} O with E = (Z[k] + conj(Z[N-k]))/2,
// O = (Z[k] - conj(Z[N-k]))/(2i), k = 0..N.
template <int N, typename T>
__device__ __forceinline__ void r2c_x_body(const FieldsT<T>& src, const FieldsT<typename Cx<T>::type>& dst,
                                           const GridDev& g, int nrows,
                                           const typename Cx<T>::type* __restrict__ tw_n,
                                           const typename Cx<T>::type* __restrict__ tw_nx, int bx, int f,
                                           typename Cx<T>::type* buf) {
    using C = typename Cx<T>::type;
    constexpr int RX = per_cta(N);
    constexpr int LD = ld_of<C>(N);
    const int row0 = bx * RX;
    const C* __restrict__ s = reinterpret_cast<const C*>(field_ptr(src, f));
    C* d = field_ptr(dst, f);
    constexpr int ITERS = RX * N / kThreads;
    static_assert((RX * N) % kThreads == 0, "rows split evenly over the threads");
    C v[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        v[it] = (row0 + r < nrows) ? s[(size_t)(row0 + r) * N + k] : mk<C>(0, 0);
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        buf[r * LD + sw<C>(k)] = v[it];
    }
    __syncthreads();
    ct_fft<N, 1, -1, RX, LD>(buf, tw_n);
    for (int t = threadIdx.x; t < RX * (N + 1); t += kThreads) {
        const int r = t / (N + 1), k = t - r * (N + 1);
        if (row0 + r < nrows) {
            const C za = buf[r * LD + sw<C>(k == N ? 0 : k)];
            const C zb = buf[r * LD + sw<C>(k == 0 ? 0 : N - k)];
            const T hf = (T)0.5;
            const C e = mk<C>(hf * (za.x + zb.x), hf * (za.y - zb.y));
            const C o = mk<C>(hf * (za.y + zb.y), -hf * (za.x - zb.x));
            const C p = cmul(__ldg(&tw_nx[k]), o);
            d[(size_t)(row0 + r) * (N + 1) + k] = mk<C>(e.x + p.x, e.y + p.y);
        }
    }
}

template <int N, typename T>
__global__ void __launch_bounds__(kThreads) k_r2c_x_ct(FieldsT<T> src, FieldsT<typename Cx<T>::type> dst,
                                                       GridDev g, int nrows,
                                                       const typename Cx<T>::type* __restrict__ tw_n,
                                                       const typename Cx<T>::type* __restrict__ tw_nx) {
    __shared__ typename Cx<T>::type buf[per_cta(N) * ld_of<typename Cx<T>::type>(N)];
    r2c_x_body<N, T>(src, dst, g, nrows, tw_n, tw_nx, blockIdx.x, blockIdx.y, buf);
}

// ------------------------------------------------------------------ fixed-point passes
// Conversions between FP64 and a transform's fixed-point grid, integer
// operations only.  A transform whose largest input has biased exponent em
// (|x| < 2^(em - 1022)) stores x as X = round(x 2^(B - em + 1022)), so that
// |X| <= 2^B, and an output X stands for X 2^(em - 1022 - B).

// Significant bits of a transform's largest input: 53, less whatever a length
// n transform (log2 n + 1 bits, the +1 for a complex modulus) and `extra` bits
// of packing growth need below 2^62.
__host__ __device__ constexpr int fx_bits(int n, int extra) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return 62 - l - 1 - extra < 53 ? 62 - l - 1 - extra : 53;
}

__device__ __forceinline__ unsigned fx_expo(double x) { return ((unsigned)__double2hiint(x) >> 20) & 0x7FFu; }
__device__ __forceinline__ unsigned fx_expo(double2 v) { return max(fx_expo(v.x), fx_expo(v.y)); }

// round(x 2^(B - em + 1022)) given rsb = 53 - B + em (em >= 1, B <= 53): the
// mantissa m of x = m 2^(ex - 1075) shifted right by rsb - ex >= 0, half up.
__device__ __forceinline__ long long fx_from(double x, int rsb) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7FF);
    const long long m = (b & 0xFFFFFFFFFFFFFLL) | (ex ? (1LL << 52) : 0LL);
    const int rs = rsb - max(ex, 1);
    long long u = 0;
    if (rs < 63) u = rs == 0 ? m : ((m >> (rs - 1)) + 1) >> 1;
    return b < 0 ? -u : u;
}

__device__ __forceinline__ double fx_to(long long X, int e2) { return i2d_scaled(X, e2); }

__device__ __forceinline__ double fx_nan() { return __longlong_as_double(0x7FF8000000000000LL); }

// emax[key] = max(emax[key], e) over the calling warp's lanes, one shared
// atomic per distinct key.  Every lane of the warp must call it.
__device__ __forceinline__ void fx_key_max(unsigned* emax, int key, unsigned e) {
    const unsigned grp = __match_any_sync(0xFFFFFFFFu, key);
    e = __reduce_max_sync(grp, e);
    if ((threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&emax[key], e);
}

// y pass in fixed point (FP64 fields); emax holds per_cta(N) exponents.
template <int N, int SIGN>
__device__ __forceinline__ void fft_y_body_fx(const Fields& src, const Fields& dst, const GridDev& g, int nplanes,
                                              int ncol, const fx2* __restrict__ tw, int bx, int f, fx2* buf,
                                              unsigned* emax) {
    constexpr int CX = per_cta(N);
    constexpr int LD = ld_of<fx2>(N);
    constexpr int B = fx_bits(N, 0);
    const long long ncols = (long long)nplanes * ncol;
    const long long vc = (long long)bx * CX + (threadIdx.x % CX);
    const bool live = vc < ncols;
    size_t base = 0;
    if (live) {
        const int p = (int)(vc / ncol);
        const int kx = (int)(vc - (long long)p * ncol);
        base = (size_t)p * g.nm + kx;
    }
    const double2* __restrict__ s = field_ptr(src, f);
    double2* d = field_ptr(dst, f);
    constexpr int ROWS_PER_ITER = kThreads / CX;
    constexpr int ITERS = N / ROWS_PER_ITER;
    static_assert(N % ROWS_PER_ITER == 0, "rows split evenly over the threads");
    const int c = threadIdx.x % CX, y0 = threadIdx.x / CX;
    if (threadIdx.x < CX) emax[threadIdx.x] = 1u;
    double2 v[ITERS];
    unsigned e = 1u;
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        v[it] = live ? s[base + (size_t)(y0 + it * ROWS_PER_ITER) * g.nxhp] : make_double2(0.0, 0.0);
        e = max(e, fx_expo(v[it]));
    }
    __syncthreads();
    fx_key_max(emax, c, e);
    __syncthreads();
    const int em = (int)emax[c];
    const int rsb = 53 - B + em;
#pragma unroll
    for (int it = 0; it < ITERS; ++it)
        buf[c * LD + sw<fx2>(y0 + it * ROWS_PER_ITER)] = mk<fx2>(fx_from(v[it].x, rsb), fx_from(v[it].y, rsb));
    __syncthreads();
    ct_fft<N, 1, SIGN, CX, LD>(buf, tw);
    if (live) {
        const int e2 = em - 1022 - B;
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const fx2 z = buf[c * LD + sw<fx2>(y0 + it * ROWS_PER_ITER)];
            d[base + (size_t)(y0 + it * ROWS_PER_ITER) * g.nxhp] =
                em == 0x7FF ? make_double2(fx_nan(), fx_nan()) : make_double2(fx_to(z.x, e2), fx_to(z.y, e2));
        }
    }
}

template <int N, int SIGN>
__global__ void __launch_bounds__(kThreads) k_fft_y_fx(Fields src, Fields dst, GridDev g, int nplanes, int ncol,
                                                       const fx2* __restrict__ tw) {
    __shared__ fx2 buf[per_cta(N) * ld_of<fx2>(N)];
    __shared__ unsigned emax[per_cta(N)];
    fft_y_body_fx<N, SIGN>(src, dst, g, nplanes, ncol, tw, blockIdx.x, blockIdx.z, buf, emax);
}

// c2r along x in fixed point: the packing of c2r_x_body (inputs of one row
// scaled together, the packing's growth of 4 within the headroom), the
// inverse transform, and the 1/(nx ny) scaling as an exact multiple of the
// FP64 constant's mantissa rounded once.
template <int N>
__device__ __forceinline__ void c2r_x_body_fx(const Fields& src, const RFields& dst, const RFields& dst2,
                                              const GridDev& g, int nrows, const fx2* __restrict__ tw_n,
                                              const fx2* __restrict__ tw_nx, int bx, int f, fx2* buf,
                                              unsigned* emax, uint64_t* mbar) {
    constexpr int RX = per_cta(N);
    constexpr int LD = ld_of<fx2>(N);
    constexpr int B = fx_bits(N, 2);
    const int row0 = bx * RX;
    const double2* __restrict__ s = field_ptr(src, f);
    double2* d = reinterpret_cast<double2*>(field_ptr(dst, f));
    double2* d2 = reinterpret_cast<double2*>(field_ptr(dst2, f));  // optional second copy (null: none)
    const int nxhp = N + 1;
    constexpr int ITERS = RX * N / kThreads;
    static_assert((RX * N) % kThreads == 0, "rows split evenly over the threads");
    if (threadIdx.x < RX) emax[threadIdx.x] = 1u;
    // The CTA's rows are contiguous in memory and the fixed-point slots are
    // as wide as a complex FP64 value, so one bulk copy (TMA engine, completion
    // on an mbarrier) stages the rows' nx/2+1 inputs into the slots as they
    // are; a copy that does not land within the wait limit marks the rows
    // non-finite.
    const int nvalid = min(RX, nrows - row0);
    if (threadIdx.x == 0) tc_mbar_init(mbar);
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)nvalid * (uint32_t)nxhp * (uint32_t)sizeof(fx2);
        tc_mbar_expect(mbar, bytes);
        tc_bulk_g2s(buf, s + (size_t)row0 * nxhp, bytes, mbar);
    }
    const bool landed = __syncthreads_and(tc_mbar_wait(mbar, 0, 1 << 22));
    unsigned e[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        fx2 ra = buf[r * LD + sw<fx2>(k)], rb = mk<fx2>(0, 0);
        if (k == 0) {  // Im of kx = 0 and kx = nx/2 is ignored
            rb = buf[r * LD + sw<fx2>(N)];
            ra.y = 0;
            rb.y = 0;
        }
        e[it] = landed ? max(fx_expo(__longlong_as_double(ra.x)), max(fx_expo(__longlong_as_double(ra.y)),
                                                                      max(fx_expo(__longlong_as_double(rb.x)),
                                                                          fx_expo(__longlong_as_double(rb.y)))))
                       : 0x7FFu;
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) fx_key_max(emax, (threadIdx.x + it * kThreads) / N, e[it]);
    __syncthreads();
    fx2 z[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        const int rsb = 53 - B + (int)emax[r];
        fx2 ra = buf[r * LD + sw<fx2>(k)], rb = buf[r * LD + sw<fx2>(N - k)];
        if (k == 0) {  // Im of kx = 0 and kx = nx/2 is ignored
            ra.y = 0;
            rb.y = 0;
        }
        const fx2 a = mk<fx2>(fx_from(__longlong_as_double(ra.x), rsb), fx_from(__longlong_as_double(ra.y), rsb));
        const fx2 b = mk<fx2>(fx_from(__longlong_as_double(rb.x), rsb), fx_from(__longlong_as_double(rb.y), rsb));
        const fx2 sm = mk<fx2>(a.x + b.x, a.y - b.y);
        const fx2 df = mk<fx2>(a.x - b.x, a.y + b.y);
        fx2 w = __ldg(&tw_nx[k]);
        w.y = -w.y;
        const fx2 p = cmul(w, df);
        z[it] = mk<fx2>(sm.x - p.y, sm.y + p.x);
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        buf[(t / N) * LD + sw<fx2>(t % N)] = z[it];
    }
    __syncthreads();
    ct_fft<N, 1, +1, RX, LD>(buf, tw_n);
    // 1/(nx ny) = M 2^(E - 1075), M its 53-bit mantissa: Y = round(Z M / 2^52)
    const long long sb = __double_as_longlong(g.inv_nxny);
    const long long M = (sb & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const int E = (int)((sb >> 52) & 0x7FF);
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        if (row0 + r < nrows) {
            const int em = (int)emax[r];
            const int e2 = em + E - 2045 - B;
            const fx2 z = buf[r * LD + sw<fx2>(k)];
            const long long yx = (long long)(((__int128)z.x * M + ((__int128)1 << 51)) >> 52);
            const long long yy = (long long)(((__int128)z.y * M + ((__int128)1 << 51)) >> 52);
            const double2 o =
                em == 0x7FF ? make_double2(fx_nan(), fx_nan()) : make_double2(fx_to(yx, e2), fx_to(yy, e2));
            d[(size_t)(row0 + r) * N + k] = o;
            if (d2) d2[(size_t)(row0 + r) * N + k] = o;
        }
    }
}

template <int N>
__global__ void __launch_bounds__(kThreads, 3) k_c2r_x_fx(Fields src, RFields dst, RFields dst2, GridDev g,
                                                          int nrows, const fx2* __restrict__ tw_n,
                                                          const fx2* __restrict__ tw_nx) {
    __shared__ fx2 buf[per_cta(N) * ld_of<fx2>(N)];
    __shared__ unsigned emax[per_cta(N)];
    __shared__ uint64_t mbar;
    c2r_x_body_fx<N>(src, dst, dst2, g, nrows, tw_n, tw_nx, blockIdx.x, blockIdx.y, buf, emax, &mbar);
}

// r2c along x in fixed point: z[m] = x[2m] + i x[2m+1] of one row scaled
// together, forward transform, and 2 X[k] = (Z[k] + conj Z[N-k]) +
// e^{-2 pi i k/nx} (-i)(Z[k] - conj Z[N-k]) formed exactly, the factor 1/2
// taken into the exponent.
template <int N>
__device__ __forceinline__ void r2c_x_body_fx(const RFields& src, const Fields& dst, const GridDev& g, int nrows,
                                              const fx2* __restrict__ tw_n, const fx2* __restrict__ tw_nx, int bx,
                                              int f, fx2* buf, unsigned* emax, uint64_t* mbar, bool bulk) {
    constexpr int RX = per_cta(N);
    constexpr int LD = N;  // rows back to back, as in memory (no kx = nx/2 slot needed)
    constexpr int B = fx_bits(N, 2);
    const int row0 = bx * RX;
    const double2* __restrict__ s = reinterpret_cast<const double2*>(field_ptr(src, f));
    double2* d = field_ptr(dst, f);
    constexpr int ITERS = RX * N / kThreads;
    static_assert((RX * N) % kThreads == 0, "rows split evenly over the threads");
    if (threadIdx.x < RX) emax[threadIdx.x] = 1u;
    // the rows' FP64 values go into the fixed-point slots as they are (z[m] =
    // x[2m] + i x[2m+1] is the row's own memory layout, and the CTA's rows are
    // contiguous): from device memory by one bulk copy (TMA engine,
    // completion on an mbarrier; a copy that does not land within the wait
    // limit marks the rows non-finite), from host memory the device maps
    // (pinned buffers read in place) by plain loads
    const int nvalid = min(RX, nrows - row0);
    bool landed = true;
    if (bulk) {
        if (threadIdx.x == 0) tc_mbar_init(mbar);
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t bytes = (uint32_t)nvalid * (uint32_t)(N * sizeof(fx2));
            tc_mbar_expect(mbar, bytes);
            tc_bulk_g2s(buf, s + (size_t)row0 * N, bytes, mbar);
        }
        landed = __syncthreads_and(tc_mbar_wait(mbar, 0, 1 << 22));
    } else {
        double2 h[ITERS];
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int t = threadIdx.x + it * kThreads;
            const int r = t / N, k = t - r * N;
            h[it] = r < nvalid ? s[(size_t)(row0 + r) * N + k] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int t = threadIdx.x + it * kThreads;
            buf[(t / N) * LD + sw<fx2>(t % N)] = mk<fx2>(__double_as_longlong(h[it].x), __double_as_longlong(h[it].y));
        }
        __syncthreads();
    }
    fx2 v[ITERS];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        v[it] = buf[r * LD + sw<fx2>(k)];
        fx_key_max(emax, r,
                   landed ? max(fx_expo(__longlong_as_double(v[it].x)), fx_expo(__longlong_as_double(v[it].y)))
                          : 0x7FFu);
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = threadIdx.x + it * kThreads;
        const int r = t / N, k = t - r * N;
        const int rsb = 53 - B + (int)emax[r];
        buf[r * LD + sw<fx2>(k)] = mk<fx2>(fx_from(__longlong_as_double(v[it].x), rsb),
                                           fx_from(__longlong_as_double(v[it].y), rsb));
    }
    __syncthreads();
    ct_fft<N, 1, -1, RX, LD>(buf, tw_n);
    for (int t = threadIdx.x; t < RX * (N + 1); t += kThreads) {
        const int r = t / (N + 1), k = t - r * (N + 1);
        if (row0 + r < nrows) {
            const fx2 za = buf[r * LD + sw<fx2>(k == N ? 0 : k)];
            const fx2 zb = buf[r * LD + sw<fx2>(k == 0 ? 0 : N - k)];
            const fx2 e = mk<fx2>(za.x + zb.x, za.y - zb.y);
            const fx2 o = mk<fx2>(za.y + zb.y, zb.x - za.x);
            const fx2 p = cmul(__ldg(&tw_nx[k]), o);
            const int em = (int)emax[r];
            const int e2 = em - 1023 - B;
            d[(size_t)(row0 + r) * (N + 1) + k] = em == 0x7FF
                                                      ? make_double2(fx_nan(), fx_nan())
                                                      : make_double2(fx_to(e.x + p.x, e2), fx_to(e.y + p.y, e2));
        }
    }
}

template <int N>
__global__ void __launch_bounds__(kThreads) k_r2c_x_fx(RFields src, Fields dst, GridDev g, int nrows,
                                                       const fx2* __restrict__ tw_n, const fx2* __restrict__ tw_nx,
                                                       int bulk) {
    __shared__ fx2 buf[per_cta(N) * ld_of<fx2>(N)];
    __shared__ unsigned emax[per_cta(N)];
    __shared__ uint64_t mbar;
    r2c_x_body_fx<N>(src, dst, g, nrows, tw_n, tw_nx, blockIdx.x, blockIdx.y, buf, emax, &mbar, bulk != 0);
}

// ------------------------------------------------------------------ ragged stages
// The four transform passes of the nonlinear term over many runs in one launch
// (k_stage, ragged.cuh): the transform length is a run property, so each CTA
// switches to the compile-time kernel body of its run's length and uses one
// shared buffer sized for the longest.
__host__ __device__ constexpr int ct_buf_max() {
    int m = 0;
#define BUF_MAX(n) m = (per_cta(n) * ld_of<float2>(n) > m) ? per_cta(n) * ld_of<float2>(n) : m;
    DNS3D_CT_Y_LENGTHS(BUF_MAX)
    DNS3D_CT_X_LENGTHS(BUF_MAX)
#undef BUF_MAX
    return m;
}

// Field f of a descriptor pointer list as field 0 of a FieldsT: the bodies
// then select field 0, and only the one pointer is held in registers.
template <typename P>
__device__ __forceinline__ FieldsT<P> one_field(void* const* p, int f) {
    FieldsT<P> r;
#pragma unroll
    for (int i = 0; i < kMaxFields; ++i) r.p[i] = nullptr;
    r.p[0] = static_cast<P*>(p[f]);
    return r;
}

// y pass: inverse over the six inputs into the scratch fields, or forward in
// place over the three sources (2/3-filtered columns only).
template <int SIGN, typename T>
struct RsFftY {
    static constexpr int kMinCtas = sizeof(T) == 8 ? 3 : 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        using C = typename Cx<T>::type;
        __shared__ C buf[ct_buf_max()];
        const int gx = d.gx[SIGN > 0 ? kRsFftYInv : kRsFftYFwd];
        const int f = b / gx, bx = b - f * gx;
        const FieldsT<C> src = one_field<C>(SIGN > 0 ? d.spec : d.src, f);
        const FieldsT<C> dst = one_field<C>(SIGN > 0 ? d.tmp : d.src, f);
        const int ncol = SIGN > 0 ? d.g.nxhp : d.ncol;
        const C* tw = static_cast<const C*>(d.tw_ny);
        switch (d.g.ny) {
#define Y_CASE(n) \
    case n: fft_y_body<n, SIGN, C>(src, dst, d.g, d.g.nz, ncol, tw, bx, 0, buf); break;
            DNS3D_CT_Y_LENGTHS(Y_CASE)
#undef Y_CASE
        }
    }
};

template <typename T>
struct RsC2R {
    static constexpr int kMinCtas = sizeof(T) == 8 ? 2 : 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        using C = typename Cx<T>::type;
        __shared__ C buf[ct_buf_max()];
        const int gx = d.gx[kRsFftC2R];
        const int f = b / gx, bx = b - f * gx;
        const C* twn = static_cast<const C*>(d.tw_nx2);
        const C* twx = static_cast<const C*>(d.tw_nx);
        switch (d.g.nxh) {
#define X_CASE(n)                                                                                              \
    case n:                                                                                                    \
        c2r_x_body<n, T>(one_field<C>(d.tmp, f), one_field<T>(d.phys, f), d.g, d.g.nz * d.g.ny, twn, twx, bx, \
                         0, buf);                                                                              \
        break;
            DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        }
    }
};

template <typename T>
struct RsR2C {
    static constexpr int kMinCtas = sizeof(T) == 8 ? 3 : 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        using C = typename Cx<T>::type;
        __shared__ C buf[ct_buf_max()];
        const int gx = d.gx[kRsFftR2C];
        const int f = b / gx, bx = b - f * gx;
        const C* twn = static_cast<const C*>(d.tw_nx2);
        const C* twx = static_cast<const C*>(d.tw_nx);
        switch (d.g.nxh) {
#define X_CASE(n)                                                                                              \
    case n:                                                                                                    \
        r2c_x_body<n, T>(one_field<T>(d.phys, f), one_field<C>(d.src, f), d.g, d.g.nz * d.g.ny, twn, twx, bx, \
                         0, buf);                                                                              \
        break;
            DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        }
    }
};

// The same passes of FP64 runs in fixed point (RunDesc twiddles: Q62 tables).
template <int SIGN>
struct RsFftYFx {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        __shared__ fx2 buf[ct_buf_max()];
        __shared__ unsigned emax[64];
        const int gx = d.gx[SIGN > 0 ? kRsFftYInv : kRsFftYFwd];
        const int f = b / gx, bx = b - f * gx;
        const Fields src = one_field<double2>(SIGN > 0 ? d.spec : d.src, f);
        const Fields dst = one_field<double2>(SIGN > 0 ? d.tmp : d.src, f);
        const int ncol = SIGN > 0 ? d.g.nxhp : d.ncol;
        const fx2* tw = static_cast<const fx2*>(d.tw_ny);
        switch (d.g.ny) {
#define Y_CASE(n) \
    case n: fft_y_body_fx<n, SIGN>(src, dst, d.g, d.g.nz, ncol, tw, bx, 0, buf, emax); break;
            DNS3D_CT_Y_LENGTHS(Y_CASE)
#undef Y_CASE
        }
    }
};

struct RsC2RFx {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        __shared__ fx2 buf[ct_buf_max()];
        __shared__ unsigned emax[64];
        __shared__ uint64_t mbar;
        const int gx = d.gx[kRsFftC2R];
        const int f = b / gx, bx = b - f * gx;
        const fx2* twn = static_cast<const fx2*>(d.tw_nx2);
        const fx2* twx = static_cast<const fx2*>(d.tw_nx);
        switch (d.g.nxh) {
#define X_CASE(n)                                                                                               \
    case n:                                                                                                     \
        c2r_x_body_fx<n>(one_field<double2>(d.tmp, f), one_field<double>(d.phys, f), RFields{}, d.g,           \
                         d.g.nz * d.g.ny, twn, twx, bx, 0, buf, emax, &mbar);                                   \
        break;
            DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        }
    }
};

struct RsR2CFx {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        __shared__ fx2 buf[ct_buf_max()];
        __shared__ unsigned emax[64];
        __shared__ uint64_t mbar;
        const int gx = d.gx[kRsFftR2C];
        const int f = b / gx, bx = b - f * gx;
        const fx2* twn = static_cast<const fx2*>(d.tw_nx2);
        const fx2* twx = static_cast<const fx2*>(d.tw_nx);
        switch (d.g.nxh) {
#define X_CASE(n)                                                                                              \
    case n:                                                                                                    \
        r2c_x_body_fx<n>(one_field<double>(d.phys, f), one_field<double2>(d.src, f), d.g, d.g.nz * d.g.ny, twn, \
                         twx, bx, 0, buf, emax, &mbar, true);                                                  \
        break;
            DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        }
    }
};

}  // namespace

int fft_ct_per_cta(int n) { return per_cta(n); }

StageKernel ragged_fft_kernel(int stage, bool mixed, bool fx) {
    if (!mixed && fx) {
        switch (stage) {
            case kRsFftYInv: return k_stage<RsFftYFx<+1>>;
            case kRsFftC2R: return k_stage<RsC2RFx>;
            case kRsFftR2C: return k_stage<RsR2CFx>;
            case kRsFftYFwd: return k_stage<RsFftYFx<-1>>;
        }
        return nullptr;
    }
    switch (stage) {
        case kRsFftYInv: return mixed ? k_stage<RsFftY<+1, float>> : k_stage<RsFftY<+1, double>>;
        case kRsFftC2R: return mixed ? k_stage<RsC2R<float>> : k_stage<RsC2R<double>>;
        case kRsFftR2C: return mixed ? k_stage<RsR2C<float>> : k_stage<RsR2C<double>>;
        case kRsFftYFwd: return mixed ? k_stage<RsFftY<-1, float>> : k_stage<RsFftY<-1, double>>;
    }
    return nullptr;
}

namespace {

template <int SIGN, typename C, int N>
void launch_y(FieldsT<C> src, FieldsT<C> dst, const GridDev& g, int nplanes, int ncol, int nf, const C* tw,
              cudaStream_t s) {
    constexpr int CX = per_cta(N);
    const long long ncols = (long long)nplanes * ncol;
    dim3 grid((unsigned)((ncols + CX - 1) / CX), 1, nf);
    k_fft_y_ct<N, SIGN, C><<<grid, kThreads, 0, s>>>(src, dst, g, nplanes, ncol, tw);
}

template <typename T, int N>
void launch_c2r(FieldsT<typename Cx<T>::type> src, FieldsT<T> dst, const GridDev& g, int nrows, int nf,
                const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s) {
    constexpr int RX = per_cta(N);
    dim3 grid((nrows + RX - 1) / RX, nf);
    k_c2r_x_ct<N, T><<<grid, kThreads, 0, s>>>(src, dst, g, nrows, tw_n, tw_nx);
}

template <typename T, int N>
void launch_r2c(FieldsT<T> src, FieldsT<typename Cx<T>::type> dst, const GridDev& g, int nrows, int nf,
                const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s) {
    constexpr int RX = per_cta(N);
    dim3 grid((nrows + RX - 1) / RX, nf);
    k_r2c_x_ct<N, T><<<grid, kThreads, 0, s>>>(src, dst, g, nrows, tw_n, tw_nx);
}

template <int SIGN, int N>
void launch_y_fx(Fields src, Fields dst, const GridDev& g, int nplanes, int ncol, int nf, const fx2* tw,
                 cudaStream_t s) {
    constexpr int CX = per_cta(N);
    const long long ncols = (long long)nplanes * ncol;
    dim3 grid((unsigned)((ncols + CX - 1) / CX), 1, nf);
    k_fft_y_fx<N, SIGN><<<grid, kThreads, 0, s>>>(src, dst, g, nplanes, ncol, tw);
}

template <int N>
void launch_c2r_fx(Fields src, RFields dst, RFields dst2, const GridDev& g, int nrows, int nf, const fx2* tw_n,
                   const fx2* tw_nx, cudaStream_t s) {
    constexpr int RX = per_cta(N);
    dim3 grid((nrows + RX - 1) / RX, nf);
    k_c2r_x_fx<N><<<grid, kThreads, 0, s>>>(src, dst, dst2, g, nrows, tw_n, tw_nx);
}

template <int N>
void launch_r2c_fx(RFields src, Fields dst, const GridDev& g, int nrows, int nf, const fx2* tw_n, const fx2* tw_nx,
                   bool host_src, cudaStream_t s) {
    constexpr int RX = per_cta(N);
    dim3 grid((nrows + RX - 1) / RX, nf);
    k_r2c_x_fx<N><<<grid, kThreads, 0, s>>>(src, dst, g, nrows, tw_n, tw_nx, host_src ? 0 : 1);
}

}  // namespace


bool fft_ct_supported(int ny, int nxh) {
    bool y = false, x = false;
#define Y_CASE(n) y = y || ny == n;
#define X_CASE(n) x = x || nxh == n;
    DNS3D_CT_Y_LENGTHS(Y_CASE)
    DNS3D_CT_X_LENGTHS(X_CASE)
#undef Y_CASE
#undef X_CASE
    return y && x;
}

template <int SIGN, typename C>
cudaError_t fft_ct_y(FieldsT<C> src, FieldsT<C> dst, const GridDev& g, int nplanes, int ncol, int nf, const C* tw,
                     cudaStream_t s) {
    if (ncol < 1 || ncol > g.nxhp) return cudaErrorInvalidValue;
    switch (g.ny) {
#define Y_CASE(n) \
    case n: launch_y<SIGN, C, n>(src, dst, g, nplanes, ncol, nf, tw, s); break;
        DNS3D_CT_Y_LENGTHS(Y_CASE)
#undef Y_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t fft_ct_c2r_x(FieldsT<typename Cx<T>::type> src, FieldsT<T> dst, const GridDev& g, int nrows, int nf,
                         const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s) {
    switch (g.nxh) {
#define X_CASE(n) \
    case n: launch_c2r<T, n>(src, dst, g, nrows, nf, tw_n, tw_nx, s); break;
        DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t fft_ct_r2c_x(FieldsT<T> src, FieldsT<typename Cx<T>::type> dst, const GridDev& g, int nrows, int nf,
                         const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s) {
    switch (g.nxh) {
#define X_CASE(n) \
    case n: launch_r2c<T, n>(src, dst, g, nrows, nf, tw_n, tw_nx, s); break;
        DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int SIGN>
cudaError_t fft_fx_y(Fields src, Fields dst, const GridDev& g, int nplanes, int ncol, int nf, const longlong2* tw,
                     cudaStream_t s) {
    if (ncol < 1 || ncol > g.nxhp) return cudaErrorInvalidValue;
    switch (g.ny) {
#define Y_CASE(n) \
    case n: launch_y_fx<SIGN, n>(src, dst, g, nplanes, ncol, nf, tw, s); break;
        DNS3D_CT_Y_LENGTHS(Y_CASE)
#undef Y_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t fft_fx_c2r_x(Fields src, RFields dst, RFields dst2, const GridDev& g, int nrows, int nf,
                         const longlong2* tw_n, const longlong2* tw_nx, cudaStream_t s) {
    switch (g.nxh) {
#define X_CASE(n) \
    case n: launch_c2r_fx<n>(src, dst, dst2, g, nrows, nf, tw_n, tw_nx, s); break;
        DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t fft_fx_r2c_x(RFields src, Fields dst, const GridDev& g, int nrows, int nf, const longlong2* tw_n,
                         const longlong2* tw_nx, bool host_src, cudaStream_t s) {
    switch (g.nxh) {
#define X_CASE(n) \
    case n: launch_r2c_fx<n>(src, dst, g, nrows, nf, tw_n, tw_nx, host_src, s); break;
        DNS3D_CT_X_LENGTHS(X_CASE)
#undef X_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template cudaError_t fft_fx_y<-1>(Fields, Fields, const GridDev&, int, int, int, const longlong2*, cudaStream_t);
template cudaError_t fft_fx_y<+1>(Fields, Fields, const GridDev&, int, int, int, const longlong2*, cudaStream_t);

template cudaError_t fft_ct_y<-1, double2>(Fields, Fields, const GridDev&, int, int, int, const double2*,
                                         cudaStream_t);
template cudaError_t fft_ct_y<+1, double2>(Fields, Fields, const GridDev&, int, int, int, const double2*,
                                         cudaStream_t);
template cudaError_t fft_ct_y<-1, float2>(FFields, FFields, const GridDev&, int, int, int, const float2*,
                                         cudaStream_t);
template cudaError_t fft_ct_y<+1, float2>(FFields, FFields, const GridDev&, int, int, int, const float2*,
                                         cudaStream_t);
template cudaError_t fft_ct_c2r_x<double>(Fields, RFields, const GridDev&, int, int, const double2*, const double2*,
                                          cudaStream_t);
template cudaError_t fft_ct_c2r_x<float>(FFields, FRFields, const GridDev&, int, int, const float2*, const float2*,
                                         cudaStream_t);
template cudaError_t fft_ct_r2c_x<double>(RFields, Fields, const GridDev&, int, int, const double2*, const double2*,
                                          cudaStream_t);
template cudaError_t fft_ct_r2c_x<float>(FRFields, FFields, const GridDev&, int, int, const float2*, const float2*,
                                         cudaStream_t);

}  // namespace dns3d

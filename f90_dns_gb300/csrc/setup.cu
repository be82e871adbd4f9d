// Per-mode operator inverses, built once per handle on the device.
//
// The reference assembles and factors an nz x nz system for every (kx, ky)
// mode at every call: the Helmholtz operator (solve_viscous_helmholtz,
// DNS_pressure_BC_3D.f90:1464-1505) and the Galerkin Poisson operator
// (solve_pressure_3d_standard, 3D:1680-1714) with zgesv.  Both depend on the
// mode only through k^2 = xsq(kx) + ysq(ky) and are constant in time, so here
// each distinct operator is inverted once (Gauss-Jordan, partial pivoting,
// FP64, one CTA per matrix in shared memory) and every step applies the
// inverse as one matrix-vector product per mode.
//
//   Helmholtz, q < nq:  A = f S + diag((1 + f k^2) w ybar/2), rows 1 and nz
//                       replaced by identity rows (3D:1480-1502)
//   Poisson,   q < nq:  P = -S - diag(k^2 w ybar/2)              (3D:1684-1692)
//   Poisson,   q = nq:  the pinned (0,0) operator: -S with row 1 and column 1
//                       zeroed and P(1,1) = 1                     (3D:1702-1711)
// Outputs are stored parity-folded per q (the operators are centro-symmetric,
// so only the two diagonal blocks of the folded inverse are non-zero), each
// block transposed; the pinned operator is not centro-symmetric and is stored
// unfolded and transposed: out[z'][z] = inverse[z][z'].
#include "dns3d_internal.cuh"
#include "tc.cuh"

namespace dns3d {
namespace {

// In-place Gauss-Jordan inversion of a[n][n] (shared memory) with partial
// pivoting; the row interchanges are undone as column interchanges at the end.
// Returns false if a zero pivot was met.
__device__ bool gj_invert(double* a, int n, int* perm, double* colk, int* flag) {
    __shared__ int piv_row;
    if (threadIdx.x == 0) *flag = 0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x < 32) {
            double best = -1.0;
            int bi = k;
            for (int i = k + threadIdx.x; i < n; i += 32) {
                const double v = fabs(a[i * n + k]);
                if (v > best) { best = v; bi = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (threadIdx.x == 0) {
                piv_row = bi;
                perm[k] = bi;
                if (!(best > 0.0)) *flag = 1;
            }
        }
        __syncthreads();
        if (*flag) return false;
        const int p = piv_row;
        if (p != k) {
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                const double t = a[k * n + j];
                a[k * n + j] = a[p * n + j];
                a[p * n + j] = t;
            }
            __syncthreads();
        }
        const double pivinv = 1.0 / a[k * n + k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) a[k * n + j] = (j == k) ? pivinv : a[k * n + j] * pivinv;
        for (int i = threadIdx.x; i < n; i += blockDim.x) colk[i] = a[i * n + k];
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int i = t / n, j = t - i * n;
            if (i == k) continue;
            const double base = (j == k) ? 0.0 : a[t];
            a[t] = base - a[k * n + j] * colk[i];
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const double t = a[i * n + k];
                a[i * n + k] = a[i * n + p];
                a[i * n + p] = t;
            }
        }
        __syncthreads();
    }
    return true;
}

// Element (i, j) of the full operator of job (helm | poisson, q).
__device__ __forceinline__ double op_elem(bool helm, int i, int j, int nz, const double* __restrict__ S,
                                          const double* __restrict__ wh, double helm_f, double k2) {
    if (helm) {
        if (i == 0 || i == nz - 1) return (i == j) ? 1.0 : 0.0;
        double v = helm_f * S[i * nz + j];
        if (i == j) v += (1.0 + helm_f * k2) * wh[i];
        return v;
    }
    double v = -S[i * nz + j];
    if (i == j) v -= k2 * wh[i];
    return v;
}

// Regular modes: the operators are centro-symmetric, so in the parity-folded
// basis they are block diagonal.  With Ae, Ao the folded blocks of A (the
// fold of step.cu) the folded blocks of A^{-1} are
//   Ge = Dm^{-1} Ae^{-1} Dm^{-1},  Dm = diag(2, ..., 2, 1 [middle, odd nz]),
//   Go = Ao^{-1} / 4,
// so each job inverts two ~nz/2 blocks instead of one nz x nz matrix.
__global__ void __launch_bounds__(256) k_build_inverses_folded(int nz, const double* __restrict__ S,
                                                               const double* __restrict__ wh, double helm_f,
                                                               const double* __restrict__ ksq, int nq,
                                                               double* __restrict__ HinvF,
                                                               double* __restrict__ PinvF, int* info) {
    extern __shared__ double sm[];
    const int h = nz / 2, he = nz - h, ho = h;
    double* ae = sm;                       // [he][he]
    double* ao = sm + he * he;             // [ho][ho]
    double* colk = ao + ho * ho;           // [he]
    int* perm = reinterpret_cast<int*>(colk + he);
    __shared__ int flag;
    const int job = blockIdx.x;  // [0, nq): Helmholtz q;  [nq, 2nq): Poisson q - nq
    const bool helm = job < nq;
    const int q = helm ? job : job - nq;
    const size_t qstride = (size_t)he * he + (size_t)ho * ho;
    double* out = (helm ? HinvF : PinvF) + (size_t)q * qstride;
    if (!helm && q == 0) {  // k^2 = 0 unpinned Poisson operator is singular and never used
        for (int t = threadIdx.x; t < (int)qstride; t += blockDim.x) out[t] = 0.0;
        return;
    }
    const double k2 = ksq[q];
    for (int t = threadIdx.x; t < he * he; t += blockDim.x) {
        const int i = t / he, j = t - i * he;
        double v;
        if (i < h && j < h) v = 0.5 * (op_elem(helm, i, j, nz, S, wh, helm_f, k2) +
                                       op_elem(helm, i, nz - 1 - j, nz, S, wh, helm_f, k2));
        else v = op_elem(helm, i, j, nz, S, wh, helm_f, k2);  // middle row / column (odd nz)
        ae[t] = v;
    }
    for (int t = threadIdx.x; t < ho * ho; t += blockDim.x) {
        const int i = t / ho, j = t - i * ho;
        ao[t] = 0.5 * (op_elem(helm, i, j, nz, S, wh, helm_f, k2) - op_elem(helm, i, nz - 1 - j, nz, S, wh, helm_f, k2));
    }
    __syncthreads();
    bool ok = gj_invert(ae, he, perm, colk, &flag);
    if (ok && ho > 0) ok = gj_invert(ao, ho, perm, colk, &flag);
    if (!ok) {
        if (threadIdx.x == 0) atomicCAS(info, 0, job + 1);
        return;
    }
    // GeT[j][k] = Ge[k][j] = ae^{-1}[k][j] / (dm_k dm_j);  GoT[j][k] = ao^{-1}[k][j] / 4
    for (int t = threadIdx.x; t < he * he; t += blockDim.x) {
        const int j = t / he, k = t - j * he;
        const double dk = (k < h) ? 2.0 : 1.0, dj = (j < h) ? 2.0 : 1.0;
        out[t] = ae[k * he + j] / (dk * dj);
    }
    for (int t = threadIdx.x; t < ho * ho; t += blockDim.x) {
        const int j = t / ho, k = t - j * ho;
        out[(size_t)he * he + t] = 0.25 * ao[k * ho + j];
    }
}

// The pinned (0,0) Poisson operator (row and column 1 zeroed, P(1,1) = 1) is
// not centro-symmetric: inverted at full size, stored unfolded and transposed.
__global__ void __launch_bounds__(256) k_build_pinned(int nz, const double* __restrict__ S,
                                                      double* __restrict__ PpinT, int* info) {
    extern __shared__ double sm[];
    double* a = sm;
    double* colk = sm + nz * nz;
    int* perm = reinterpret_cast<int*>(colk + nz);
    __shared__ int flag;
    for (int t = threadIdx.x; t < nz * nz; t += blockDim.x) {
        const int i = t / nz, j = t - i * nz;
        a[t] = (i == 0 || j == 0) ? ((i == 0 && j == 0) ? 1.0 : 0.0) : -S[t];
    }
    __syncthreads();
    if (!gj_invert(a, nz, perm, colk, &flag)) {
        if (threadIdx.x == 0) atomicCAS(info, 0, 1);
        return;
    }
    for (int t = threadIdx.x; t < nz * nz; t += blockDim.x) {
        const int zp = t / nz, z = t - zp * nz;
        PpinT[t] = a[z * nz + zp];
    }
}

// Eight independent FMA chains per thread; one store per thread keeps the
// chains live.
__global__ void __launch_bounds__(256) k_fma_probe(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = threadIdx.x + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Digit slices of the folded inverses for the tensor-core solve (tc.cuh):
// one thread per (q, row of the block-diagonal operator).  Row i of the even
// block is Ge[i][:] = GeT[:][i], entered with its columns scaled by 2 w_j
// (G'[i][j] = 2 w_j G[i][j], w the folded quadrature weights: the kernel's
// right-hand sides are the weight-free halves of the folded ones).  Rows i of
// the even and the odd block share one exponent (the larger of the two rows'
// scales), so that the kernel can form x_i = xe_i + xo_i and x_nz-1-i =
// xe_i - xo_i exactly in integers.  Rows and columns past a block's size
// stay zero, so the padded core matrices contribute nothing.
__global__ void k_tc_slices(const double* __restrict__ invF, const double* __restrict__ wfold, int nq, int nz,
                            __half* __restrict__ slices, int* __restrict__ rowexp) {
    const TcGeom t = tc_geom(nz);
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)nq * t.m8) return;
    const int q = (int)(id / t.m8), m = (int)(id - (long long)q * t.m8);
    const bool even = m < t.e8;
    const int i = even ? m : m - t.e8;
    const int n = even ? t.he : t.ho;
    const int w8 = even ? t.e8 : t.o8;
    const size_t qs = (size_t)t.he * t.he + (size_t)t.ho * t.ho;
    const double* GeT = invF + (size_t)q * qs;
    const double* GoT = GeT + (size_t)t.he * t.he;
    const double* GT = even ? GeT : GoT;
    __half* S = slices + (size_t)q * tc_q_halves(t);
    const int ncore = t.ncore_e + t.ncore_o;
    const int cbase = even ? 0 : t.ncore_e;
    const int nb = w8 / 8;
    int e = 0;
    if (i < n) {
        unsigned long long mx = 0;
        auto scan = [&](const double* G, int len) {
            for (int j = 0; j < len; ++j) {
                const double v = 2.0 * wfold[j] * G[(size_t)j * len + i];
                const unsigned long long ab = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
                mx = ab > mx ? ab : mx;
            }
        };
        scan(GeT, t.he);
        if (i < t.ho) scan(GoT, t.ho);
        e = tc_exponent(mx);
    }
    rowexp[(size_t)q * t.m8 + m] = e;
    for (int j = 0; j < w8; ++j) {
        int c[kTcSlices];
        for (int s = 0; s < kTcSlices; ++s) c[s] = 0;
        if (i < n && j < n) tc_digits(tc_fixed(2.0 * wfold[j] * GT[(size_t)j * n + i], e), c);
        const int core = cbase + (i / 8) * nb + (j / 8);
        const int off = (i % 8) * 8 + (j % 8);
        for (int s = 0; s < kTcSlices; ++s) S[((size_t)s * ncore + core) * 64 + off] = __int2half_rn(c[s]);
    }
}

// Digit image of the folded antisymmetric operator [[0, De], [Do, 0]] (the
// z-derivative on [fe; fo]) in the two-block layout of tc.cuh, whole (zeros
// included: it is staged once per CTA): per digit, block E = De (e8 rows x ko
// K) then block O = Do (o8 rows x ke K); rowexp [m8] (even rows first).  One
// thread per row.
__global__ void k_tc_anti_image(const double* __restrict__ De, const double* __restrict__ Do, int nz,
                                __half* __restrict__ image, int* __restrict__ rowexp) {
    const TcGeom t = tc_geom(nz);
    const TcBlocks bl = tc_blocks(t, true);
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= t.m8) return;
    const bool even = m < t.e8;
    const int i = even ? m : m - t.e8;
    const int n = even ? t.ho : t.he;          // row length (K of the block)
    const int kw = even ? bl.kE : bl.kO;       // padded K width of the block
    const bool live = i < (even ? t.he : t.ho);
    const double* row = even ? De + (size_t)i * t.ho : Do + (size_t)i * t.he;
    const size_t base = even ? 0 : (size_t)bl.aE;
    int e = 0;
    if (live) {
        unsigned long long mx = 0;
        for (int j = 0; j < n; ++j) {
            const unsigned long long ab = (unsigned long long)__double_as_longlong(row[j]) & 0x7FFFFFFFFFFFFFFFULL;
            mx = ab > mx ? ab : mx;
        }
        e = tc_exponent(mx);
    }
    rowexp[m] = e;
    for (int j = 0; j < kw; ++j) {
        int c[kTcSlices];
        for (int s = 0; s < kTcSlices; ++s) c[s] = 0;
        if (live && j < n) tc_digits(tc_fixed(row[j], e), c);
        for (int s = 0; s < kTcSlices; ++s)
            image[(size_t)s * bl.a + base + tc_core_off(i, j, kw)] = __int2half_rn(c[s]);
    }
}

// One thread per (q, folded row): the row's exponent e (smallest with
// |G[k][j]| < 2^e over the row) and its entries as round(G 2^(58 - e)).
__global__ void k_fixed_rows(const double* __restrict__ GF, int nq, int he, int ho, long long* __restrict__ GI,
                             int* __restrict__ GE) {
    const int nr = he + ho;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nq * nr) return;
    const int q = (int)(t / nr), r = (int)(t - (long long)q * nr);
    const bool even = r < he;
    const int n = even ? he : ho, k = even ? r : r - he;
    const size_t src = (size_t)q * ((size_t)he * he + (size_t)ho * ho) + (even ? 0 : (size_t)he * he);
    const size_t dst = (size_t)q * fx_qstride(he, ho) + (even ? 0 : (size_t)he * he);
    unsigned long long mx = 0;
    for (int j = 0; j < n; ++j) {
        const unsigned long long ab = (unsigned long long)__double_as_longlong(GF[src + (size_t)j * n + k]) &
                                      0x7FFFFFFFFFFFFFFFULL;
        mx = ab > mx ? ab : mx;
    }
    const int e = tc_exponent(mx);
    GE[t] = e;
    for (int j = 0; j < n; ++j) GI[dst + (size_t)j * n + k] = tc_fixed_bits<58>(GF[src + (size_t)j * n + k], e);
}

}  // namespace

cudaError_t build_tc_anti_image(const GridDev& g, const double* De, const double* Do, __half* image, int* rowexp,
                                cudaStream_t s) {
    const TcGeom t = tc_geom(g.nz);
    k_tc_anti_image<<<(t.m8 + 127) / 128, 128, 0, s>>>(De, Do, g.nz, image, rowexp);
    return cudaGetLastError();
}

cudaError_t build_tc_slices(const GridDev& g, const double* invF, const double* wfold, int nq, __half* slices,
                            int* rowexp, cudaStream_t s) {
    const TcGeom t = tc_geom(g.nz);
    const long long n = (long long)nq * t.m8;
    k_tc_slices<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(invF, wfold, nq, g.nz, slices, rowexp);
    return cudaGetLastError();
}

cudaError_t measure_fp64_tflops(int device, double* tflops) {
    cudaError_t e;
    if ((e = cudaSetDevice(device))) return e;
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device))) return e;
    const int blocks = sms * 8, threads = 256, iters = 4000;
    double* out = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double) * blocks * threads))) return e;
    cudaStream_t s;
    cudaEvent_t e0, e1;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_probe<<<blocks, threads, 0, s>>>(out, 64, 0.999, 0.001);
    double best = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, s);
        k_fma_probe<<<blocks, threads, 0, s>>>(out, iters, 0.999, 0.001);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        if (e) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double tf = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
        if (tf > best) best = tf;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    *tflops = best;
    return e ? e : cudaGetLastError();
}

cudaError_t build_inverses(const GridDev& g, const double* S, const double* wh, double helm_f,
                           const double* ksq, int nq, double* HinvF, double* PinvF, double* PpinT, int* info,
                           cudaStream_t s) {
    const int nz = g.nz, h = nz / 2, he = nz - h, ho = h;
    const size_t sm_f = ((size_t)he * he + (size_t)ho * ho + he) * sizeof(double) + he * sizeof(int);
    const size_t sm_p = ((size_t)nz * nz + nz) * sizeof(double) + nz * sizeof(int);
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev))) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k_build_inverses_folded))) return e;
    int limit = optin - (int)fa.sharedSizeBytes;
    if ((int)sm_f > limit) return cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute(k_build_inverses_folded, cudaFuncAttributeMaxDynamicSharedMemorySize, limit)))
        return e;
    if ((e = cudaFuncGetAttributes(&fa, k_build_pinned))) return e;
    limit = optin - (int)fa.sharedSizeBytes;
    if ((int)sm_p > limit) return cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute(k_build_pinned, cudaFuncAttributeMaxDynamicSharedMemorySize, limit))) return e;
    k_build_inverses_folded<<<2 * nq, 256, sm_f, s>>>(nz, S, wh, helm_f, ksq, nq, HinvF, PinvF, info);
    k_build_pinned<<<1, 256, sm_p, s>>>(nz, S, PpinT, info);
    return cudaGetLastError();
}

cudaError_t build_fixed_rows(const GridDev& g, const double* PinvF, int nq, long long* PinvI, int* PinvE,
                             cudaStream_t s) {
    const int ho = g.nz / 2, he = g.nz - ho;
    const long long n = (long long)nq * (he + ho);
    k_fixed_rows<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(PinvF, nq, he, ho, PinvI, PinvE);
    return cudaGetLastError();
}

}  // namespace dns3d

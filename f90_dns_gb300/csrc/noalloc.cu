// Flow statistics of caller-owned device fields without any device allocation.
//
// Who needs this: programs that own every byte of device memory themselves --
// for example a driver that reserves nearly all HBM for its own pool at start-up
// and then must not see a library allocate behind its back, or a caller whose
// memory budget is fixed per job -- cannot use dns3d_diagnostics(), because that
// needs a handle whose creation allocates device buffers.  This entry point
// computes the same max|u|, max|v|, max|w| and kinetic energy as
// dns3d_diagnostics() from u, v, w arrays the caller already holds on the
// device, and writes the four numbers to a caller-owned device buffer.
//
// Its only scratch (one partial result per thread block) lives in the
// file-scope array below, which exists once per GPU that loads this library and
// stays allocated until the process exits.  Nothing here calls cudaMalloc,
// cudaFree or any other allocating routine.
#include <cmath>
#include <mutex>
#include <vector>

#include "dns3d_internal.cuh"

namespace {

constexpr int kBlocks = 1024;   // thread blocks of the partial pass
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// Per-block partials: [kBlocks][4] = max|u|, max|v|, max|w|, sum 0.5|u|^2 w_k.
// Every call overwrites the kBlocks*4 entries it reads, so nothing has to start
// at zero; two calls that overlap on the GPU share this array and race.
static __device__ __align__(256) double g_stats_scratch[kBlocks * 4];

std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};

struct Weights {
    double w[DNS3D_NOALLOC_MAX_NZ];
};

// LGL quadrature weights of n nodes from the library's own setup routine
// (lgl_nodes_weights, lgl_module.f90:30-80), copied into the by-value kernel
// argument.  The host vector is host memory; no device memory is allocated.
void lgl_weights_fixed(int n, Weights& out) {
    std::vector<double> x, w;
    dns3d::lgl_nodes_weights(n, x, w);
    for (int i = 0; i < n; ++i) out.w[i] = w[i];
}

// max that keeps a NaN: once either operand is NaN the result is NaN, so a
// non-finite field shows up in out4[0..2] (the fmax builtin would drop it).
__device__ __forceinline__ double nanmax(double m, double a) { return (a != a || a > m) ? a : m; }

__device__ __forceinline__ double wmax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads) k_stats_partial(const double* __restrict__ u,
                                                            const double* __restrict__ v,
                                                            const double* __restrict__ w, size_t plane,
                                                            size_t n, Weights zw, double* __restrict__ part) {
    double mu = 0.0, mv = 0.0, mw = 0.0, e = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double a = u[i], b = v[i], c = w[i];
        mu = nanmax(mu, fabs(a));
        mv = nanmax(mv, fabs(b));
        mw = nanmax(mw, fabs(c));
        e += 0.5 * (a * a + b * b + c * c) * zw.w[i / plane];
    }
    __shared__ double red[4][kThreads / 32];
    mu = wmax(mu); mv = wmax(mv); mw = wmax(mw); e = wsum(e);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { red[0][wid] = mu; red[1][wid] = mv; red[2][wid] = mw; red[3][wid] = e; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kThreads / 32; ++k) {
            mu = nanmax(mu, red[0][k]); mv = nanmax(mv, red[1][k]); mw = nanmax(mw, red[2][k]); e += red[3][k];
        }
        part[4 * blockIdx.x + 0] = mu;
        part[4 * blockIdx.x + 1] = mv;
        part[4 * blockIdx.x + 2] = mw;
        part[4 * blockIdx.x + 3] = e;
    }
}

__global__ void k_stats_final(const double* __restrict__ part, double scale, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double mu = 0.0, mv = 0.0, mw = 0.0, e = 0.0;
    for (int b = 0; b < kBlocks; ++b) {
        mu = nanmax(mu, part[4 * b]);
        mv = nanmax(mv, part[4 * b + 1]);
        mw = nanmax(mw, part[4 * b + 2]);
        e += part[4 * b + 3];
    }
    out[0] = mu;
    out[1] = mv;
    out[2] = mw;
    out[3] = e * scale;
}

// Device address of g_stats_scratch on the current device, looked up once per
// device.  A host-side reference to g_stats_scratch names a host stand-in, not
// device memory, so kernels must be given this address instead.  The cache is
// keyed by device ordinal for the life of the process: it does not survive
// cudaDeviceReset() or a switch to another context on the same device (the
// module is loaded again there, at another address).
int scratch_address(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return DNS3D_E_NODEVICE;
    if (dev >= kMaxDevices) return DNS3D_E_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_stats_scratch);
        if (e != cudaSuccess || !p) return DNS3D_E_CUDA;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return DNS3D_OK;
}

}  // namespace

extern "C" int dns3d_flow_stats_noalloc(const double* u, const double* v, const double* w, int nx, int ny,
                                        int nz, double* out4, void* stream) {
    if (!u || !v || !w || !out4 || nx < 1 || ny < 1) return DNS3D_E_INVALID;
    if (nz < 2 || nz > DNS3D_NOALLOC_MAX_NZ) return DNS3D_E_UNSUPPORTED;
    double* part = nullptr;
    int rc = scratch_address(&part);
    if (rc) return rc;
    Weights zw{};
    lgl_weights_fixed(nz, zw);
    const size_t plane = (size_t)nx * ny;
    const size_t n = plane * (size_t)nz;
    // energy = sum 0.5|u|^2 w_k (Lx/nx)(Ly/ny)(ybar/2) / (Lx Ly ybar) with ybar = 2
    // (DNS_pressure_BC_3D.f90:2110-2128) = sum 0.5|u|^2 w_k / (2 nx ny)
    const double scale = 1.0 / (2.0 * (double)nx * (double)ny);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_stats_partial<<<kBlocks, kThreads, 0, s>>>(u, v, w, plane, n, zw, part);
    k_stats_final<<<1, 32, 0, s>>>(part, scale, out4);
    return cudaGetLastError() == cudaSuccess ? DNS3D_OK : DNS3D_E_CUDA;
}

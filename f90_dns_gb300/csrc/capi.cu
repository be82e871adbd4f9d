// C-ABI entry points of libdns3d_gpu.so (declared in include/dns3d_capi.h).
//
// The handle owns the device state of one channel run: the spectra of u, v,
// w and p_total, the wall planes of grad(p_total) the next step's Kim & Moin
// boundary condition reads, the PI controller state, the LGL operators and
// the per-mode operator inverses.  The five stage entry points run the same
// kernels that dns3d_step() captures into a CUDA graph.
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "dns3d_internal.cuh"
#include "ragged.cuh"
#include "tc.cuh"

using namespace dns3d;

struct dns3d_handle {
    dns3d_config cfg{};
    GridDev g{};
    cudaStream_t stream = nullptr;
    // A second stream for work off the critical path (the PI update during the
    // nonlinear term; the FP64 mean-mode solves of the mixed form beside their
    // FP32 mode tiles), forked from and joined back to `stream` by events.
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev[3] = {nullptr, nullptr, nullptr}, join_ev[3] = {nullptr, nullptr, nullptr};
    FftCtx fft{};
    Ops ops{};
    MixedOps mx{};
    bool mixed = false;
    float2* spec32[6] = {nullptr};  // mixed: u, v, w, ox, oy, oz (FP32 spectra)
    float2* src32[3] = {nullptr};   // mixed: nonlinear source spectra
    float* phys32[6] = {nullptr};   // mixed: physical planes
    StepParams sp{};
    PIParams pp{};
    double2 *U = nullptr, *V = nullptr, *W = nullptr, *P = nullptr, *GP = nullptr;
    double2 *SU = nullptr, *SV = nullptr, *SW = nullptr;
    double2 *US = nullptr, *VS = nullptr, *WS = nullptr, *PHI = nullptr;
    double2* PHIZ = nullptr;  // mixed: dphi/dz
    double2* RK[3] = {nullptr, nullptr, nullptr};  // jst4 stage state (convection_scheme 1)
    double* phys[6] = {nullptr};
    dns3d_pi_state* d_pi = nullptr;
    double* d_red = nullptr;
    double* d_out = nullptr;
    double* h_out = nullptr;  // pinned host copy of d_out (the diagnostics' one read-back)
    int* d_flag = nullptr;
    int* d_tcerr = nullptr;  // [2]: set when a tensor-core completion wait ran out
    // viscous solve on the tensor cores (ops.tcA built): chosen by the tile
    // autotuner unless DNS3D_TENSOR_CORES forces it (1) or rules it out (0)
    bool visc_tc = false;
    bool visc_tc_forced = false;
    // the vorticity's and the projection's z-derivatives on the tensor cores
    // (ops.tcD built), chosen likewise
    bool vort_tc = false;
    bool corr_tc = false;
    bool pres_tc = false;  // the strong-form pressure right-hand side's D1.w*
    int red_blocks = 0;
    std::vector<double> zpts, zwts;
    std::vector<void*> allocs;
    int step = 0;
    double time = 0.0;
    cudaGraphExec_t graph = nullptr;
    std::string err;
    // profiling marks: an event recorded after every kernel launch
    bool prof = false;
    std::vector<cudaEvent_t> ev;
    std::vector<const char*> evname;
    size_t nev = 0;
    int launches = 0;  // kernel launches of the last step body
    // Bit f set: phys[f] holds the physical field f (u, v, w, p_total) of the
    // current state, left by get_state or diagnostics.  Everything that changes
    // the state or reuses phys[] as scratch clears it.
    unsigned phys_valid = 0;
    // set_state / get_state read and write pinned host buffers in place from
    // the transform kernels (DNS3D_ZERO_COPY=0 turns this off)
    bool zero_copy = true;
};

namespace {

constexpr double kPi = 3.14159265358979323846;  // 4*atan(1), DNS_pressure_BC_3D.f90:43

int cuda_fail(dns3d_handle* h, cudaError_t e, const char* what) {
    if (h) {
        h->err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return (e == cudaErrorMemoryAllocation) ? DNS3D_E_OOM : DNS3D_E_CUDA;
}

#define CK(h, call)                                              \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
    } while (0)

template <typename T>
int dev_alloc(dns3d_handle* h, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) > 0 ? count * sizeof(T) : 1);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
    h->allocs.push_back(q);
    // every buffer starts zeroed (work buffers are read by the tile autotuner)
    e = h->stream ? cudaMemsetAsync(q, 0, count * sizeof(T), h->stream) : cudaMemset(q, 0, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemset");
    *p = static_cast<T*>(q);
    return DNS3D_OK;
}

size_t spec_elems(const dns3d_config& c) { return (size_t)(c.nx / 2 + 1) * c.ny * c.nz; }
size_t phys_elems(const dns3d_config& c) { return (size_t)c.nx * c.ny * c.nz; }
int n_unique_q(const dns3d_config& c) { return (c.ny / 2 + 1) * (c.nx / 2 + 1); }

int validate(const dns3d_config* c) {
    if (!c) return DNS3D_E_INVALID;
    if (c->nx < 4 || c->ny < 4 || (c->nx % 2) || (c->ny % 2)) return DNS3D_E_UNSUPPORTED;
    if (!fft_length_supported(c->ny) || !fft_length_supported(c->nx / 2)) return DNS3D_E_UNSUPPORTED;
    if (c->nx > 1024 || c->ny > 1024) return DNS3D_E_UNSUPPORTED;
    if (c->nz < 3 || c->nz > 129) return DNS3D_E_UNSUPPORTED;
    if (!(c->dt > 0.0) || !(c->re > 0.0) || !(c->xlen > 0.0) || !(c->ylen > 0.0)) return DNS3D_E_INVALID;
    // parameter validation of read_input_3d (3D:649-679)
    if (c->flow_control_method != 1 && c->flow_control_method != 2) return DNS3D_E_INVALID;
    if (c->flow_control_method == 2) {
        if (!(c->target_bulk_velocity > 0.0) || !(c->controller_gain > 0.0) || c->controller_update_freq <= 0)
            return DNS3D_E_INVALID;
    }
    if (c->precision != DNS3D_PREC_FP64 && c->precision != DNS3D_PREC_MIXED) return DNS3D_E_UNSUPPORTED;
    if (c->convection_scheme != 0 && c->convection_scheme != 1) return DNS3D_E_INVALID;
    if (c->linear_solver != 0 && c->linear_solver != 1) return DNS3D_E_INVALID;
    if (c->linear_solver == 1 && !(c->cgstol > 0.0)) return DNS3D_E_INVALID;
    if (c->linear_solver == 1 && c->precision != DNS3D_PREC_FP64) return DNS3D_E_UNSUPPORTED;
    if (!(c->noise_amplitude >= 0.0)) return DNS3D_E_INVALID;
    if (c->poisson_refinement != 0 && c->poisson_refinement != 1) return DNS3D_E_INVALID;
    return DNS3D_OK;
}

// Physical initial condition of initialize_fields_3d (3D:909-962) with
// generate_analytical_perturbations (perturbation_analytical_simple.f90:24-155).
void initial_fields(const dns3d_config& c, const std::vector<double>& z, std::vector<double>& u,
                    std::vector<double>& v, std::vector<double>& w) {
    const int nx = c.nx, ny = c.ny, nz = c.nz;
    const size_t pl = (size_t)nx * ny;
    u.assign(pl * nz, 0.0);
    v.assign(pl * nz, 0.0);
    w.assign(pl * nz, 0.0);
    for (int k = 0; k < nz; ++k)
        for (size_t i = 0; i < pl; ++i) u[k * pl + i] = c.u_centerline * (1.0 - z[k] * z[k]);
    if (!c.enable_perturbations || !c.use_analytical_perturbations) return;
    const double kx = 2.0 * kPi * (double)c.analytical_mode_x / c.xlen;
    const double ky = 2.0 * kPi * (double)c.analytical_mode_y / c.ylen;
    std::vector<double> up(pl * nz), vp(pl * nz);
    double cur = 0.0;
    for (int k = 0; k < nz; ++k) {
        const double damp = 1.0 - z[k] * z[k];
        for (int j = 0; j < ny; ++j) {
            const double y = (double)j * c.ylen / (double)ny;
            for (int i = 0; i < nx; ++i) {
                const double x = (double)i * c.xlen / (double)nx;
                const size_t o = k * pl + (size_t)j * nx + i;
                up[o] = -ky * std::sin(kx * x) * std::cos(ky * y) * damp;
                vp[o] = kx * std::cos(kx * x) * std::sin(ky * y) * damp;
                const double mag = std::sqrt(up[o] * up[o] + vp[o] * vp[o]);
                if (mag > cur) cur = mag;
            }
        }
    }
    if (cur > 1.0e-12) {  // scale_perturbations (:110-133)
        const double s = c.perturbation_amplitude / cur;
        for (size_t o = 0; o < pl * nz; ++o) { up[o] *= s; vp[o] *= s; }
    } else {
        std::fill(up.begin(), up.end(), 0.0);
        std::fill(vp.begin(), vp.end(), 0.0);
    }
    for (size_t o = 0; o < pl * nz; ++o) { u[o] += up[o]; v[o] += vp[o]; }
    for (int k : {0, nz - 1})  // enforce_wall_boundaries + apply_boundary_conditions_3d (3D:3253)
        for (size_t i = 0; i < pl; ++i) { u[k * pl + i] = 0.0; v[k * pl + i] = 0.0; w[k * pl + i] = 0.0; }
}

// SplitMix64 (Steele, Lea and Flood, OOPSLA 2014; the finaliser constants
// of Stafford's Mix13): output i is mix(seed + (i+1) * 0x9E3779B97F4A7C15);
// a uniform double in [0, 1) takes its top 53 bits.
struct SplitMix64 {
    uint64_t s;
    double uniform() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * 0x1.0p-53;
    }
};

// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11): ten rounds of
// (c0, c1, c2, c3) -> (hi(B c2) ^ c1 ^ k0, lo(B c2), hi(A c0) ^ c3 ^ k1, lo(A c0))
// with A = 0xD2511F53, B = 0xCD9E8D57 and the key bumped by the Weyl
// constants (0x9E3779B9, 0xBB67AE85) between rounds.
void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

// The white-noise sample of component comp at point n (C order k, j, i).
double noise_sample(uint64_t seed, uint64_t n, int comp, double amplitude) {
    uint32_t c[4] = {(uint32_t)n, (uint32_t)(n >> 32), (uint32_t)comp, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t a = c[0] >> 5, b = c[1] >> 6;  // 27 + 26 bits
    const double u = (double)(a * 67108864ull + b) * 0x1.0p-53;
    return amplitude * (2.0 * u - 1.0);
}

// integrate_with_boundary_conditions_fallback (perturbation_module.f90:
// 470-517): trapezoid integral of -div upward from w(-1) = 0, a quadratic
// correction that brings w(+1) to zero, and sin^2 tapers on the three
// levels next to each wall (with the reference's 3.14159).
void integrate_w_column(int nz, const double* z, const double* div, double* w) {
    std::vector<double> up(nz);
    up[0] = 0.0;
    for (int k = 1; k < nz; ++k) up[k] = up[k - 1] - 0.5 * (div[k] + div[k - 1]) * (z[k] - z[k - 1]);
    const double total = up[nz - 1];
    for (int k = 0; k < nz; ++k) {
        const double zn = (z[k] - z[0]) / (z[nz - 1] - z[0]);
        w[k] = up[k] - total * (zn * (2.0 - zn));
    }
    w[0] = 0.0;
    w[nz - 1] = 0.0;
    for (int k = 2; k <= std::min(4, nz - 1); ++k) {  // Fortran levels
        const double s = std::sin(0.5 * 3.14159 * (double)(k - 1) / 3.0);
        w[k - 1] *= s * s;
    }
    for (int k = std::max(nz - 3, 2); k <= nz - 1; ++k) {
        const double s = std::sin(0.5 * 3.14159 * (double)(nz - k) / 3.0);
        w[k - 1] *= s * s;
    }
}

void mark(dns3d_handle* h, const char* name) {
    h->launches += 1;
    if (!h->prof) return;
    if (h->nev == h->ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        h->ev.push_back(e);
        h->evname.push_back(nullptr);
    }
    cudaEventRecord(h->ev[h->nev], h->stream);
    h->evname[h->nev] = name;
    h->nev += 1;
}

void fft_hook(void* ctx, const char* name) { mark(static_cast<dns3d_handle*>(ctx), name); }

// Side-branch work: launched on h->side after everything queued so far on
// h->stream, and joined back before the next dependent launch.  While the
// kernels are being profiled one by one the branch stays on h->stream, so
// each event pair brackets exactly one kernel.
cudaStream_t side_stream(dns3d_handle* h) { return h->prof ? h->stream : h->side; }

cudaError_t fork_side(dns3d_handle* h, int i) {
    if (h->prof) return cudaSuccess;
    cudaError_t e = cudaEventRecord(h->fork_ev[i], h->stream);
    return e ? e : cudaStreamWaitEvent(h->side, h->fork_ev[i], 0);
}

cudaError_t join_side(dns3d_handle* h, int i) {
    if (h->prof) return cudaSuccess;
    cudaError_t e = cudaEventRecord(h->join_ev[i], h->side);
    return e ? e : cudaStreamWaitEvent(h->stream, h->join_ev[i], 0);
}

// Parity folding of a full row-major operator (see step.cu): antisymmetric
// D -> De [he][ho], Do [ho][he]; symmetric A -> Ae [he][he], Ao [ho][ho].
void fold_antisymmetric(const std::vector<double>& D, int n, std::vector<double>& De, std::vector<double>& Do) {
    const int h = n / 2, he = n - h, ho = h;
    De.assign((size_t)he * ho, 0.0);
    Do.assign((size_t)ho * he, 0.0);
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < h; ++j) {
            De[(size_t)i * ho + j] = 0.5 * (D[(size_t)i * n + j] - D[(size_t)i * n + n - 1 - j]);
            Do[(size_t)i * he + j] = 0.5 * (D[(size_t)i * n + j] + D[(size_t)i * n + n - 1 - j]);
        }
        if (n % 2) Do[(size_t)i * he + h] = D[(size_t)i * n + h];
    }
    if (n % 2)
        for (int j = 0; j < h; ++j) De[(size_t)h * ho + j] = D[(size_t)h * n + j];
}

void fold_symmetric(const std::vector<double>& A, int n, std::vector<double>& Ae, std::vector<double>& Ao) {
    const int h = n / 2, he = n - h, ho = h;
    Ae.assign((size_t)he * he, 0.0);
    Ao.assign((size_t)ho * ho, 0.0);
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < h; ++j) {
            Ae[(size_t)i * he + j] = 0.5 * (A[(size_t)i * n + j] + A[(size_t)i * n + n - 1 - j]);
            Ao[(size_t)i * ho + j] = 0.5 * (A[(size_t)i * n + j] - A[(size_t)i * n + n - 1 - j]);
        }
        if (n % 2) Ae[(size_t)i * he + h] = A[(size_t)i * n + h];
    }
    if (n % 2) {
        for (int j = 0; j < h; ++j) Ae[(size_t)h * he + j] = A[(size_t)h * n + j];
        Ae[(size_t)h * he + h] = A[(size_t)h * n + h];
    }
}

// The device address of host memory that kernels can read and write in
// place: pinned memory (cudaHostAlloc, cudaHostRegister), which the unified
// address space maps for the device -- on this machine over NVLink-C2C.
// Null for pageable memory, which goes through copies.
double* device_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<double*>(a.devicePointer);
}

int upload(dns3d_handle* h, void* dst, const void* src, size_t bytes) {
    CK(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
    return DNS3D_OK;
}

// The nonlinear term of the velocity spectra in[0..2] (the state, or a jst4
// stage state): FP32 sources in src32 (mixed) or FP64 sources in SU..SW.
int run_source_terms_mixed(dns3d_handle* h, double2* const* in) {
    const GridDev& g = h->g;
    FFields sp{};
    for (int f = 0; f < 6; ++f) sp.p[f] = h->spec32[f];
    CK(h, launch_vorticity_mixed(g, h->mx, h->ops, in[0], in[1], in[2], sp, h->stream));
    mark(h, "vorticity32");
    FRFields ph{};
    for (int f = 0; f < 6; ++f) ph.p[f] = h->phys32[f];
    CK(h, fft_c2r32(h->fft, g, sp, ph, 6, g.nz, h->stream));
    FRFields prod{};
    for (int f = 0; f < 3; ++f) prod.p[f] = h->phys32[f];
    CK(h, launch_products32(g, ph, prod, h->stream));
    mark(h, "products32");
    FFields src{};
    for (int f = 0; f < 3; ++f) src.p[f] = h->src32[f];
    // the 2/3 filter discards kx > kx_max: those columns skip the y pass
    CK(h, fft_r2c32(h->fft, g, prod, src, 3, g.nz, h->stream, h->sp.dealias ? h->sp.kx_max + 1 : 0));
    return DNS3D_OK;
}

int run_source_terms_fp64(dns3d_handle* h, double2* const* in);

int run_source_terms(dns3d_handle* h) {
    h->phys_valid = 0;
    const GridDev& g = h->g;
    // the PI update reads only the mean mode of u and writes only the
    // controller state, which the viscous step reads: it runs beside the
    // nonlinear term and joins at the end of this stage
    CK(h, fork_side(h, 0));
    CK(h, launch_pi_update(g, h->ops, h->pp, h->U, h->d_pi, side_stream(h)));
    mark(h, "pi_update");
    double2* state[3] = {h->U, h->V, h->W};
    double2* const* in = state;
    int rc;
    if (h->cfg.convection_scheme == 1) {
        // jst4 (DNS_pressure_BC_2D.f90:931-1014 lifted to 3D): three stage
        // states u^n + (1/irk) dt S(previous), irk = 4, 3, 2; the step's
        // source is S of the last one
        Fields F{}, R{};
        for (int f = 0; f < 3; ++f) { F.p[f] = state[f]; R.p[f] = h->RK[f]; }
        for (int irk = 4; irk >= 2; --irk) {
            rc = h->mixed ? run_source_terms_mixed(h, in) : run_source_terms_fp64(h, in);
            if (rc) return rc;
            const double coef = (1.0 / (double)irk) * h->cfg.dt;
            if (h->mixed) {
                FFields S{};
                for (int f = 0; f < 3; ++f) S.p[f] = h->src32[f];
                CK(h, launch_rk_stage(g, h->sp, coef, F, S, R, h->stream));
            } else {
                Fields S{};
                S.p[0] = h->SU; S.p[1] = h->SV; S.p[2] = h->SW;
                CK(h, launch_rk_stage(g, h->sp, coef, F, S, R, h->stream));
            }
            mark(h, "jst4_stage");
            in = h->RK;
        }
    }
    rc = h->mixed ? run_source_terms_mixed(h, in) : run_source_terms_fp64(h, in);
    if (rc) return rc;
    CK(h, join_side(h, 0));
    return DNS3D_OK;
}

int run_source_terms_fp64(dns3d_handle* h, double2* const* in) {
    const GridDev& g = h->g;
    // u, v, w to physical space on the side stream while the vorticity runs:
    // they need only the state, and the vorticity kernel leaves SMs free
    // (scratch slots 0-2 and phys[0..2] here, 3-5 and phys[3..5] below)
    CK(h, fork_side(h, 1));
    {
        Fields su{};
        RFields pu{};
        for (int f = 0; f < 3; ++f) {
            su.p[f] = in[f];
            pu.p[f] = h->phys[f];
        }
        CK(h, fft_c2r(h->fft, g, su, pu, 3, g.nz, side_stream(h), 0));
    }
    // vorticity into the u*,v*,w* buffers (free until the viscous step)
    if (h->vort_tc) {
        CK(h, launch_vorticity_tc(g, h->ops, in[0], in[1], in[2], h->US, h->VS, h->WS, h->d_tcerr, h->stream));
        mark(h, "vorticity_tc");
    } else {
        CK(h, launch_vorticity(g, h->ops, in[0], in[1], in[2], h->US, h->VS, h->WS, h->stream));
        mark(h, "vorticity");
    }
    Fields spec{};
    spec.p[0] = h->US; spec.p[1] = h->VS; spec.p[2] = h->WS;
    RFields phys{};
    for (int f = 0; f < 3; ++f) phys.p[f] = h->phys[3 + f];
    CK(h, fft_c2r(h->fft, g, spec, phys, 3, g.nz, h->stream, 3));
    CK(h, join_side(h, 1));
    RFields all{};  // u, v, w, ox, oy, oz in physical space
    for (int f = 0; f < 6; ++f) all.p[f] = h->phys[f];
    RFields prod{};
    for (int f = 0; f < 3; ++f) prod.p[f] = h->phys[f];
    CK(h, launch_products(g, all, prod, h->stream));
    mark(h, "products");
    Fields src{};
    src.p[0] = h->SU; src.p[1] = h->SV; src.p[2] = h->SW;
    // the 2/3 filter discards kx > kx_max: those columns skip the y pass
    CK(h, fft_r2c(h->fft, g, prod, src, 3, g.nz, h->stream, h->sp.dealias ? h->sp.kx_max + 1 : 0));
    return DNS3D_OK;
}

int run_viscous(dns3d_handle* h) {
    h->phys_valid = 0;
    if (h->mixed) {
        Fields F{}, O{};
        FFields S{};
        F.p[0] = h->U; F.p[1] = h->V; F.p[2] = h->W;
        O.p[0] = h->US; O.p[1] = h->VS; O.p[2] = h->WS;
        for (int f = 0; f < 3; ++f) S.p[f] = h->src32[f];
        // mode (0,0) in FP64 on the side branch, all other modes in FP32 tiles
        CK(h, fork_side(h, 1));
        CK(h, launch_viscous_mean_mode(h->g, h->ops, h->sp, F, S, h->GP, h->d_pi, O, side_stream(h)));
        mark(h, "viscous_mean_mode");
        CK(h, launch_viscous_mixed(h->g, h->mx, h->ops, h->sp, F, S, h->GP, O, h->stream));
        mark(h, "viscous_mixed");
        CK(h, join_side(h, 1));
        return DNS3D_OK;
    }
    Fields F{}, S{}, O{};
    F.p[0] = h->U; F.p[1] = h->V; F.p[2] = h->W;
    S.p[0] = h->SU; S.p[1] = h->SV; S.p[2] = h->SW;
    O.p[0] = h->US; O.p[1] = h->VS; O.p[2] = h->WS;
    if (h->cfg.linear_solver == 1) {  // jacgs on the right-hand sides
        StepParams sr = h->sp;
        sr.rhs_only = 1;
        CK(h, launch_viscous(h->g, h->ops, sr, F, S, h->GP, h->d_pi, O, h->stream));
        mark(h, "viscous_rhs");
        CK(h, launch_pcg_helmholtz(h->g, h->ops, h->sp, O, h->cfg.cgstol, h->stream));
        mark(h, "viscous_jacgs");
        return DNS3D_OK;
    }
    if (h->visc_tc && h->ops.tcA && h->sp.cn_identity) {
        CK(h, launch_viscous_tc(h->g, h->ops, h->sp, F, S, h->GP, h->d_pi, O, h->d_tcerr, h->stream));
        mark(h, "viscous_helmholtz_tc");
        return DNS3D_OK;
    }
    CK(h, launch_viscous(h->g, h->ops, h->sp, F, S, h->GP, h->d_pi, O, h->stream));
    mark(h, "viscous_helmholtz");
    return DNS3D_OK;
}

int run_pressure(dns3d_handle* h) {
    h->phys_valid = 0;
    if (h->mixed) {
        CK(h, fork_side(h, 2));
        CK(h, launch_pressure_mean_mode(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->PHIZ, side_stream(h)));
        mark(h, "pressure_mean_mode");
        CK(h, launch_pressure_mixed(h->g, h->mx, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->PHIZ, h->stream));
        mark(h, "pressure_mixed");
        CK(h, join_side(h, 2));
        return DNS3D_OK;
    }
    if (h->cfg.linear_solver == 1) {  // jacgs; the pinned (0,0) mode stays direct
        StepParams sr = h->sp;
        sr.rhs_only = 1;
        CK(h, launch_pressure(h->g, h->ops, sr, h->US, h->VS, h->WS, h->PHI, h->stream));
        mark(h, "pressure_rhs");
        CK(h, launch_pcg_poisson(h->g, h->ops, h->PHI, h->cfg.cgstol, h->stream));
        mark(h, "pressure_jacgs");
        return DNS3D_OK;
    }
    if (h->pres_tc) {
        CK(h, launch_pressure_tc(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->d_tcerr, h->stream));
        mark(h, "pressure_poisson_tc");
        return DNS3D_OK;
    }
    CK(h, launch_pressure(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->stream));
    mark(h, "pressure_poisson");
    return DNS3D_OK;
}

// pressure_correction_3d; with fuse_bc the projection also writes the wall
// planes of u, v, w as apply_boundary_conditions_3d does (the fused step)
int run_correction(dns3d_handle* h, bool fuse_bc = false) {
    h->phys_valid = 0;
    StepParams sp = h->sp;
    sp.bc_walls = fuse_bc ? 1 : 0;
    if (h->mixed) {
        CK(h, launch_correction_mixed(h->g, h->ops, sp, h->US, h->VS, h->WS, h->PHI, h->PHIZ, h->U, h->V, h->W,
                                      h->P, h->GP, h->stream));
        mark(h, "correction_mixed");
        return DNS3D_OK;
    }
    if (h->corr_tc) {
        CK(h, launch_correction_tc(h->g, h->ops, sp, h->US, h->VS, h->WS, h->PHI, h->U, h->V, h->W, h->P,
                                   h->GP, h->d_tcerr, h->stream));
        mark(h, "pressure_correction_tc");
        return DNS3D_OK;
    }
    CK(h, launch_correction(h->g, h->ops, sp, h->US, h->VS, h->WS, h->PHI, h->U, h->V, h->W, h->P,
                            h->GP, h->stream));
    mark(h, "pressure_correction");
    return DNS3D_OK;
}

int run_bc(dns3d_handle* h) {
    h->phys_valid = 0;
    CK(h, launch_apply_bc(h->g, h->U, h->V, h->W, h->stream));
    mark(h, "apply_bc");
    return DNS3D_OK;
}

int run_step_body(dns3d_handle* h) {
    int rc;
    h->launches = 0;
    h->fft.hook = fft_hook;
    h->fft.hook_ctx = h;
    if ((rc = run_source_terms(h))) return rc;
    if ((rc = run_viscous(h))) return rc;
    if ((rc = run_pressure(h))) return rc;
    // apply_boundary_conditions_3d in the projection's pass
    return run_correction(h, true);
}

void release(dns3d_handle* h) {
    if (!h) return;
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (cudaEvent_t e : h->ev) cudaEventDestroy(e);
    for (int i = 0; i < 3; ++i) {
        if (h->fork_ev[i]) cudaEventDestroy(h->fork_ev[i]);
        if (h->join_ev[i]) cudaEventDestroy(h->join_ev[i]);
    }
    if (h->side) cudaStreamDestroy(h->side);
    h->ev.clear();
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    fft_release(h->fft);
    if (h->h_out) cudaFreeHost(h->h_out);
    h->h_out = nullptr;
    if (h->stream) cudaStreamDestroy(h->stream);
}

}  // namespace

extern "C" {

int dns3d_config_defaults(dns3d_config* c) {
    if (!c) return DNS3D_E_INVALID;
    std::memset(c, 0, sizeof(*c));
    c->nx = 128; c->ny = 32; c->nz = 33;
    c->istart = 0; c->nsteps = 1000; c->nwrt = 100; c->restart_write_freq = 1000;
    c->dt = 0.01; c->re = 180.0;
    c->xlen = 2.0 * kPi; c->ylen = 2.0 * kPi;
    c->u_centerline = 1.5;
    c->use_crank_nicolson = 1;
    c->flow_control_method = 1;
    c->target_pressure_gradient = 0.03;
    c->target_bulk_velocity = 1.0;
    c->controller_gain = 0.15;
    c->controller_update_freq = 7;
    c->enable_perturbations = 0;
    c->perturbation_amplitude = 0.01;
    c->zero_w_perturbations = 0;
    c->use_analytical_perturbations = 0;
    c->analytical_mode_x = 1; c->analytical_mode_y = 1;
    c->use_weak_form_divergence = 0;
    c->use_dealias_23_rule = 0;
    c->lgl_dmatrix_guard = 1;
    c->precision = DNS3D_PREC_FP64;
    c->device = 0;
    c->perturbation_seed = 0;
    c->convection_scheme = 0;
    c->linear_solver = 0;
    c->cgstol = 1.0e-6;  // 3D:575
    c->noise_amplitude = 0.0;
    c->poisson_refinement = 0;
    c->pad_ = 0;
    return DNS3D_OK;
}

int dns3d_config_read_namelist(const char* path, dns3d_config* cfg) {
    if (!path || !cfg) return DNS3D_E_INVALID;
    return read_namelist_file(path, cfg);
}

int dns3d_footprint_bytes(const dns3d_config* c, unsigned long long* bytes) {
    if (!c || !bytes) return DNS3D_E_INVALID;
    const size_t se = spec_elems(*c), pe = phys_elems(*c);
    const size_t nm = (size_t)(c->nx / 2 + 1) * c->ny;
    const size_t nq = (size_t)n_unique_q(*c);
    const size_t nz2 = (size_t)c->nz * c->nz;
    size_t b = 0;
    b += 11 * se * sizeof(double2);          // U V W P SU SV SW US VS WS PHI
    if (c->convection_scheme == 1) b += 3 * se * sizeof(double2);  // jst4 stage state
    b += 4 * nm * sizeof(double2);           // GP
    b += 6 * se * sizeof(double2);           // FFT scratch
    b += 6 * pe * sizeof(double);            // physical fields
    const size_t hz = (size_t)c->nz / 2, ez = (size_t)c->nz - hz;
    b += (2 * nq * (ez * ez + hz * hz) + 2 * nz2) * sizeof(double);  // folded inverses, pinned, S
    if (c->precision == DNS3D_PREC_MIXED)
        b += (6 + 3 + 6) * se * sizeof(float2) + 6 * pe * sizeof(float) + se * sizeof(double2);  // + dphi/dz
    else if (tc_supported(c->nz)) {
        const TcGeom t = tc_geom(c->nz);
        if (c->use_crank_nicolson && c->linear_solver == 0)  // digit slices of the Helmholtz inverses
            b += nq * (tc_q_halves(t) * sizeof(__half) + (size_t)t.m8 * sizeof(int));
        b += (size_t)kTcSlices * tc_blocks(t, true).a * sizeof(__half);  // digit image of D1
        if (!c->use_weak_form_divergence)  // fixed-point Poisson inverses and row exponents
            b += nq * (fx_qstride((int)ez, (int)hz) * sizeof(long long) + (size_t)c->nz * sizeof(int));
    }
    b += 16ull << 20;                        // operators, tables, reductions
    *bytes = b;
    return DNS3D_OK;
}

}  // extern "C"

namespace {

// ------------------------------------------------------------------ autotuner
// Tile widths (mode columns per CTA) of the mode-tile kernels a handle runs,
// chosen by timing each candidate width on the handle's own buffers (one
// warm launch, then three between events on the handle's stream) and kept per
// (grid, precision, device) for the process, so ensembles and the server tune
// each grid once.  A width changes only the schedule: every output is one
// thread's fixed-order sum, so results are bitwise the same for any width.
using TuneKey = std::tuple<int, int, int, int, int>;
std::mutex g_tune_mu;
// the widths, then 1 if the viscous solve, the vorticity, the projection, the
// pressure right-hand side runs on the tensor cores
std::map<TuneKey, std::array<int, kTileKernels + 4>> g_tune;

int tile_launch(dns3d_handle* h, int k) {
    const GridDev& g = h->g;
    Fields F{}, S{}, O{}, T{};
    F.p[0] = h->U; F.p[1] = h->V; F.p[2] = h->W;
    S.p[0] = h->SU; S.p[1] = h->SV; S.p[2] = h->SW;
    O.p[0] = h->US; O.p[1] = h->VS; O.p[2] = h->WS;
    const size_t se = spec_elems(h->cfg);
    for (int f = 0; f < 5; ++f) T.p[f] = h->fft.tmp + (size_t)f * se;  // scratch for outputs that are state
    FFields S32{};
    for (int f = 0; f < 6; ++f) S32.p[f] = h->spec32[f];
    FFields src32{};
    for (int f = 0; f < 3; ++f) src32.p[f] = h->src32[f];
    cudaError_t e = cudaSuccess;
    switch (k) {
        case kTileVort: e = launch_vorticity(g, h->ops, h->U, h->V, h->W, h->US, h->VS, h->WS, h->stream); break;
        case kTileVisc: e = launch_viscous(g, h->ops, h->sp, F, S, h->GP, h->d_pi, O, h->stream); break;
        case kTilePres: e = launch_pressure(g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->stream); break;
        case kTileCorr:
            e = launch_correction(g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, T.p[0], T.p[1], T.p[2], T.p[3],
                                  T.p[4], h->stream);
            break;
        case kTileVortM: e = launch_vorticity_mixed(g, h->mx, h->ops, h->U, h->V, h->W, S32, h->stream); break;
        case kTileViscM: e = launch_viscous_mixed(g, h->mx, h->ops, h->sp, F, src32, h->GP, O, h->stream); break;
        case kTilePresM:
            e = launch_pressure_mixed(g, h->mx, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->PHIZ, h->stream);
            break;
        default: return DNS3D_E_INVALID;
    }
    CK(h, e);
    return DNS3D_OK;
}

int autotune(dns3d_handle* h, bool force) {
    CK(h, cudaSetDevice(h->cfg.device));
    // precision, and for FP64 whether the tensor-core solve exists / is forced
    const int variant = h->mixed ? 1 + 8 * h->g.refine : (h->ops.tcA || h->ops.tcD ? (h->visc_tc_forced ? 4 : 2) : 0);
    const TuneKey key{h->cfg.nx, h->cfg.ny, h->cfg.nz, variant, h->cfg.device};
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            for (int k = 0; k < kTileKernels; ++k) h->g.tc[k] = it->second[k];
            if (h->ops.tcA && !h->visc_tc_forced) h->visc_tc = it->second[kTileKernels] != 0;
            if (h->ops.tcD && !h->visc_tc_forced) {
                h->vort_tc = it->second[kTileKernels + 1] != 0;
                h->corr_tc = it->second[kTileKernels + 2] != 0;
                h->pres_tc = it->second[kTileKernels + 3] != 0;
            }
            return DNS3D_OK;
        }
    }
    static const int kFp64[] = {kTileVort, kTilePres, kTileCorr, kTileVisc};
    static const int kMixed[] = {kTileVortM, kTileViscM, kTilePresM};
    const int* ks = h->mixed ? kMixed : kFp64;
    // the FP64-pipe viscous kernel (last in kFp64) is not timed when the
    // tensor-core one is forced
    const int nk = h->mixed ? 3 : (h->visc_tc_forced ? 3 : 4);
    float visc_ms = 0.f, vort_ms = 0.f, corr_ms = 0.f, pres_ms = 0.f;
    cudaEvent_t e0, e1;
    CK(h, cudaEventCreate(&e0));
    CK(h, cudaEventCreate(&e1));
    int rc = DNS3D_OK;
    for (int i = 0; i < nk && !rc; ++i) {
        const int k = ks[i];
        int best = 0;
        float best_ms = 0.f;
        for (int cand : {4, 8, 16, 32, 64}) {
            if (!tile_fits(h->g, k, cand)) continue;
            h->g.tc[k] = cand;
            if ((rc = tile_launch(h, k))) break;
            cudaEventRecord(e0, h->stream);
            for (int r = 0; r < 3 && !rc; ++r) rc = tile_launch(h, k);
            cudaEventRecord(e1, h->stream);
            if (rc) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) { rc = cuda_fail(h, cudaGetLastError(), "autotune"); break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (best == 0 || ms < best_ms) { best = cand; best_ms = ms; }
        }
        h->g.tc[k] = best;  // 0 (heuristic) if no candidate fitted
        if (k == kTileVisc) visc_ms = best_ms;
        if (k == kTileVort) vort_ms = best_ms;
        if (k == kTileCorr) corr_ms = best_ms;
        if (k == kTilePres) pres_ms = best_ms;
    }
    // the tensor-core viscous solve against the best FP64-pipe width
    if (!rc && !h->mixed && h->ops.tcA && !h->visc_tc_forced) {
        Fields F{}, S{}, O{};
        F.p[0] = h->U; F.p[1] = h->V; F.p[2] = h->W;
        S.p[0] = h->SU; S.p[1] = h->SV; S.p[2] = h->SW;
        O.p[0] = h->US; O.p[1] = h->VS; O.p[2] = h->WS;
        auto launch = [&] { return launch_viscous_tc(h->g, h->ops, h->sp, F, S, h->GP, h->d_pi, O, h->d_tcerr, h->stream); };
        cudaError_t ce = launch();
        if (!ce) ce = cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 3 && !ce; ++r) ce = launch();
        if (!ce) ce = cudaEventRecord(e1, h->stream);
        if (!ce) ce = cudaEventSynchronize(e1);
        if (ce) {
            rc = cuda_fail(h, ce, "autotune (tensor-core viscous)");
        } else {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            h->visc_tc = visc_ms <= 0.f || ms < visc_ms;
        }
    }
    // the tensor-core vorticity against the best FP64-pipe width
    if (!rc && !h->mixed && h->ops.tcD && !h->visc_tc_forced) {
        auto launch = [&] {
            return launch_vorticity_tc(h->g, h->ops, h->U, h->V, h->W, h->US, h->VS, h->WS, h->d_tcerr, h->stream);
        };
        cudaError_t ce = launch();
        if (!ce) ce = cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 3 && !ce; ++r) ce = launch();
        if (!ce) ce = cudaEventRecord(e1, h->stream);
        if (!ce) ce = cudaEventSynchronize(e1);
        if (ce) {
            rc = cuda_fail(h, ce, "autotune (tensor-core vorticity)");
        } else {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            h->vort_tc = vort_ms <= 0.f || ms < vort_ms;
        }
    }
    // the tensor-core projection against the best FP64-pipe width (outputs
    // that are state go to scratch, as in tile_launch)
    if (!rc && !h->mixed && h->ops.tcD && !h->visc_tc_forced) {
        const size_t se = spec_elems(h->cfg);
        double2* T[5];
        for (int f = 0; f < 5; ++f) T[f] = h->fft.tmp + (size_t)f * se;
        auto launch = [&] {
            return launch_correction_tc(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, T[0], T[1], T[2], T[3],
                                        T[4], h->d_tcerr, h->stream);
        };
        cudaError_t ce = launch();
        if (!ce) ce = cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 3 && !ce; ++r) ce = launch();
        if (!ce) ce = cudaEventRecord(e1, h->stream);
        if (!ce) ce = cudaEventSynchronize(e1);
        if (ce) {
            rc = cuda_fail(h, ce, "autotune (tensor-core projection)");
        } else {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            h->corr_tc = corr_ms <= 0.f || ms < corr_ms;
        }
    }
    // the tensor-core pressure (right-hand side and solve) against the best
    // FP64-pipe width; the strong form only
    if (!rc && !h->mixed && h->ops.tcD && !h->visc_tc_forced && !h->sp.weak_form) {
        auto launch = [&] {
            return launch_pressure_tc(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, h->d_tcerr, h->stream);
        };
        cudaError_t ce = launch();
        if (!ce) ce = cudaEventRecord(e0, h->stream);
        for (int r = 0; r < 3 && !ce; ++r) ce = launch();
        if (!ce) ce = cudaEventRecord(e1, h->stream);
        if (!ce) ce = cudaEventSynchronize(e1);
        if (ce) {
            rc = cuda_fail(h, ce, "autotune (tensor-core pressure)");
        } else {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            h->pres_tc = pres_ms <= 0.f || ms < pres_ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    h->phys_valid = 0;  // the timing launches reused work buffers
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    std::array<int, kTileKernels + 4> tiles{};
    for (int k = 0; k < kTileKernels; ++k) tiles[k] = h->g.tc[k];
    tiles[kTileKernels] = h->visc_tc ? 1 : 0;
    tiles[kTileKernels + 1] = h->vort_tc ? 1 : 0;
    tiles[kTileKernels + 2] = h->corr_tc ? 1 : 0;
    tiles[kTileKernels + 3] = h->pres_tc ? 1 : 0;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = tiles;
    return DNS3D_OK;
}

}  // namespace

extern "C" {

int dns3d_autotune(dns3d_handle* h, int force, int* tiles, int ntiles) {
    if (!h || ntiles < 0 || (ntiles > 0 && !tiles)) return DNS3D_E_INVALID;
    if (force >= 0) {
        const int rc = autotune(h, force != 0);
        if (rc) return rc;
    }
    for (int k = 0; k < ntiles && k < kTileKernels; ++k) tiles[k] = tile_width(h->g, k);
    return DNS3D_OK;
}

int dns3d_set_tiles(dns3d_handle* h, const int* tiles, int ntiles) {
    if (!h || !tiles || ntiles < 0) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    for (int k = 0; k < ntiles && k < kTileKernels; ++k)
        if (tiles[k] != 0 && !tile_fits(h->g, k, tiles[k])) return DNS3D_E_INVALID;
    for (int k = 0; k < ntiles && k < kTileKernels; ++k) h->g.tc[k] = tiles[k];
    if (h->graph) {
        CK(h, cudaStreamSynchronize(h->stream));
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    return DNS3D_OK;
}

int dns3d_create(const dns3d_config* cfg, dns3d_handle** out) {
    if (!out) return DNS3D_E_INVALID;
    *out = nullptr;
    int rc = validate(cfg);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DNS3D_E_NODEVICE;
    if (cfg->device < 0 || cfg->device >= ndev) return DNS3D_E_INVALID;
    dns3d_handle* h = new dns3d_handle();
    h->cfg = *cfg;
    const dns3d_config& c = h->cfg;
    auto fail = [&](int code) { release(h); delete h; return code; };
    if (cudaSetDevice(c.device) != cudaSuccess) return fail(DNS3D_E_CUDA);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess)
        return fail(DNS3D_E_CUDA);
    for (int i = 0; i < 3; ++i)
        if (cudaEventCreateWithFlags(&h->fork_ev[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->join_ev[i], cudaEventDisableTiming) != cudaSuccess)
            return fail(DNS3D_E_CUDA);

    GridDev& g = h->g;
    g.nx = c.nx; g.ny = c.ny; g.nz = c.nz;
    g.nxh = c.nx / 2; g.nxhp = c.nx / 2 + 1; g.nm = g.nxhp * c.ny;
    g.nkyu = c.ny / 2 + 1;
    g.inv_nxny = 1.0 / ((double)c.nx * (double)c.ny);
    g.refine = (c.precision == DNS3D_PREC_MIXED && c.poisson_refinement) ? 1 : 0;
    const int nz = c.nz;

    // setup_grid_3d (3D:740-742) and setup_spectral_3d (3D:769-809)
    const double ybar = 2.0;
    const double zs = 2.0 / ybar;
    const double alpha = 2.0 * kPi / c.xlen;
    std::vector<double> xw(g.nxhp), yw(c.ny);
    for (int i = 0; i < g.nxhp; ++i) xw[i] = (double)i * alpha;
    for (int j = 1; j <= c.ny; ++j)
        yw[j - 1] = (j <= c.ny / 2 + 1) ? (double)(j - 1) * 2.0 * kPi / c.ylen
                                        : (double)(j - 1 - c.ny) * 2.0 * kPi / c.ylen;
    std::vector<double> d1, d2((size_t)nz * nz, 0.0);
    lgl_nodes_weights(nz, h->zpts, h->zwts);
    lgl_diff_matrix(h->zpts, c.lgl_dmatrix_guard != 0, d1);
    for (int i = 0; i < nz; ++i)  // d2 = matmul(d1, d1) (3D:801)
        for (int j = 0; j < nz; ++j) {
            double s = 0.0;
            for (int k = 0; k < nz; ++k) s += d1[(size_t)i * nz + k] * d1[(size_t)k * nz + j];
            d2[(size_t)i * nz + j] = s;
        }
    // stiffness S_kn = sum_m d1(m,k) d1(m,n) zwts(m) (2/ybar)  (3D:1467-1471)
    std::vector<double> S((size_t)nz * nz);
    for (int k = 0; k < nz; ++k)
        for (int n = 0; n < nz; ++n) {
            double s = 0.0;
            for (int m = 0; m < nz; ++m) s += d1[(size_t)m * nz + k] * d1[(size_t)m * nz + n] * h->zwts[m];
            S[(size_t)k * nz + n] = s * (2.0 / ybar);
        }
    const double theta = c.use_crank_nicolson ? 0.5 : 1.0;
    const double helm_f = theta * c.dt / c.re;
    std::vector<double> D1s((size_t)nz * nz), D2s((size_t)nz * nz), wh(nz), S0(nz), Sn(nz),
        W1T((size_t)nz * nz);
    for (size_t t = 0; t < (size_t)nz * nz; ++t) { D1s[t] = zs * d1[t]; D2s[t] = zs * zs * d2[t]; }
    for (int k = 0; k < nz; ++k) {
        wh[k] = h->zwts[k] * (ybar / 2.0);
        S0[k] = helm_f * S[(size_t)k * nz + 0];
        Sn[k] = helm_f * S[(size_t)k * nz + nz - 1];
        for (int m = 0; m < nz; ++m) W1T[(size_t)k * nz + m] = d1[(size_t)m * nz + k] * h->zwts[m] * (2.0 / ybar);
    }
    const int nq = n_unique_q(c);
    std::vector<double> ksq(nq);
    for (int kya = 0; kya <= c.ny / 2; ++kya)
        for (int kx = 0; kx < g.nxhp; ++kx) ksq[(size_t)kya * g.nxhp + kx] = xw[kx] * xw[kx] + yw[kya] * yw[kya];
    std::vector<double> D1e, D1o, D2e, D2o, W1e, W1o;
    fold_antisymmetric(D1s, nz, D1e, D1o);
    fold_symmetric(D2s, nz, D2e, D2o);
    fold_antisymmetric(W1T, nz, W1e, W1o);

    Ops& ops = h->ops;
    ops.nq = nq;
    ops.ho = nz / 2;
    ops.he = nz - ops.ho;
    const size_t nz2 = (size_t)nz * nz;
    const size_t qstride = (size_t)ops.he * ops.he + (size_t)ops.ho * ops.ho;
    double* dS = nullptr;
    if ((rc = dev_alloc(h, &ops.D1e, D1e.size())) || (rc = dev_alloc(h, &ops.D1o, D1o.size())) ||
        (rc = dev_alloc(h, &ops.D2e, D2e.size())) || (rc = dev_alloc(h, &ops.D2o, D2o.size())) ||
        (rc = dev_alloc(h, &ops.W1e, W1e.size())) || (rc = dev_alloc(h, &ops.W1o, W1o.size())) ||
        (rc = dev_alloc(h, &ops.wh, nz)) || (rc = dev_alloc(h, &ops.zw, nz)) ||
        (rc = dev_alloc(h, &ops.S0, nz)) || (rc = dev_alloc(h, &ops.Sn, nz)) ||
        (rc = dev_alloc(h, &ops.xw, g.nxhp)) || (rc = dev_alloc(h, &ops.yw, c.ny)) ||
        (rc = dev_alloc(h, &ops.ksq, nq)) || (rc = dev_alloc(h, &dS, nz2)) ||
        (rc = dev_alloc(h, &ops.HinvF, (size_t)nq * qstride)) ||
        (rc = dev_alloc(h, &ops.PinvF, (size_t)nq * qstride)) || (rc = dev_alloc(h, &ops.PpinT, nz2)))
        return fail(rc);
    struct Up { void* d; const void* s; size_t b; } ups[] = {
        {ops.D1e, D1e.data(), D1e.size() * 8}, {ops.D1o, D1o.data(), D1o.size() * 8},
        {ops.D2e, D2e.data(), D2e.size() * 8}, {ops.D2o, D2o.data(), D2o.size() * 8},
        {ops.W1e, W1e.data(), W1e.size() * 8}, {ops.W1o, W1o.data(), W1o.size() * 8},
        {ops.wh, wh.data(), (size_t)nz * 8}, {ops.zw, h->zwts.data(), (size_t)nz * 8},
        {ops.S0, S0.data(), (size_t)nz * 8}, {ops.Sn, Sn.data(), (size_t)nz * 8},
        {ops.xw, xw.data(), (size_t)g.nxhp * 8}, {ops.yw, yw.data(), (size_t)c.ny * 8},
        {ops.ksq, ksq.data(), (size_t)nq * 8}, {dS, S.data(), nz2 * 8}};
    for (auto& u : ups)
        if ((rc = upload(h, u.d, u.s, u.b))) return fail(rc);
    ops.S = dS;

    // state and work buffers
    const size_t se = spec_elems(c), pe = phys_elems(c);
    double2** specs[] = {&h->U, &h->V, &h->W, &h->P, &h->SU, &h->SV, &h->SW, &h->US, &h->VS, &h->WS, &h->PHI};
    for (auto p : specs)
        if ((rc = dev_alloc(h, p, se))) return fail(rc);
    if ((rc = dev_alloc(h, &h->GP, (size_t)4 * g.nm))) return fail(rc);
    if (c.convection_scheme == 1)
        for (int f = 0; f < 3; ++f)
            if ((rc = dev_alloc(h, &h->RK[f], se))) return fail(rc);
    for (int f = 0; f < 6; ++f)
        if ((rc = dev_alloc(h, &h->phys[f], pe))) return fail(rc);
    h->fft.tmp_fields = 6;
    if ((rc = dev_alloc(h, &h->fft.tmp, 6 * se))) return fail(rc);
    if ((rc = dev_alloc(h, &h->d_pi, 1))) return fail(rc);
    h->red_blocks = 152 * 4;
    if ((rc = dev_alloc(h, &h->d_red, (size_t)4 * h->red_blocks))) return fail(rc);
    if ((rc = dev_alloc(h, &h->d_out, 16 + 6 * (size_t)c.nz))) return fail(rc);
    if (cudaMallocHost(&h->h_out, (16 + 6 * (size_t)c.nz) * sizeof(double)) != cudaSuccess) return fail(DNS3D_E_OOM);
    if ((rc = dev_alloc(h, &h->d_flag, 4))) return fail(rc);

    cudaError_t e;
    if ((e = fft_setup(h->fft, g)) != cudaSuccess) { cuda_fail(h, e, "fft_setup"); return fail(DNS3D_E_CUDA); }
    if ((e = prepare_step_kernels(g)) != cudaSuccess) { cuda_fail(h, e, "prepare"); return fail(DNS3D_E_CUDA); }

    // per-mode operator inverses
    if (cudaMemsetAsync(h->d_flag, 0, 4 * sizeof(int), h->stream) != cudaSuccess) return fail(DNS3D_E_CUDA);
    if ((e = build_inverses(g, dS, ops.wh, helm_f, ops.ksq, nq, ops.HinvF, ops.PinvF, ops.PpinT, h->d_flag,
                            h->stream)))
        return fail(DNS3D_E_CUDA);
    int info = 0;
    if (cudaMemcpyAsync(&info, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return fail(DNS3D_E_CUDA);
    if (info != 0) return fail(DNS3D_E_SINGULAR);

    if (c.precision == DNS3D_PREC_MIXED) {
        h->mixed = true;
        // eigenbasis of the interior Helmholtz problem, S_II V = M_II V Lambda, in
        // the orthogonal even/odd basis of the (centro-symmetric) interior levels:
        // C = M^-1/2 S_II M^-1/2 splits into Ce (even) and Co (odd).
        const int ni = nz - 2, hoi = ni / 2, hei = ni - hoi;
        const int pe4 = (hei + 3) / 4 * 4, po4 = (hoi + 3) / 4 * 4;
        const double r2 = std::sqrt(2.0);
        auto Cint = [&](int i, int j) { return S[(size_t)(i + 1) * nz + (j + 1)] / std::sqrt(wh[i + 1] * wh[j + 1]); };
        std::vector<double> Ce((size_t)hei * hei), Co((size_t)hoi * hoi), le, lo, Ye, Yo;
        for (int i = 0; i < hei; ++i)
            for (int j = 0; j < hei; ++j) {
                double v;
                if (i < hoi && j < hoi) v = Cint(i, j) + Cint(i, ni - 1 - j);
                else if (i < hoi) v = r2 * Cint(i, hoi);   // middle column
                else if (j < hoi) v = r2 * Cint(hoi, j);   // middle row
                else v = Cint(hoi, hoi);
                Ce[(size_t)i * hei + j] = v;
            }
        for (int i = 0; i < hoi; ++i)
            for (int j = 0; j < hoi; ++j) Co[(size_t)i * hoi + j] = Cint(i, j) - Cint(i, ni - 1 - j);
        jacobi_eigen(hei, Ce, le, Ye);
        if (hoi > 0) jacobi_eigen(hoi, Co, lo, Yo);
        auto sq = [&](int i) { return std::sqrt(wh[i + 1]); };  // sqrt(m_i), interior index i
        std::vector<float> AeT((size_t)hei * pe4, 0.f), AoT((size_t)hoi * po4, 0.f), BeT((size_t)hei * pe4, 0.f),
            BoT((size_t)hoi * po4, 0.f), lamf(pe4 + po4, 0.f), s0f(pe4 + po4, 0.f), snf(pe4 + po4, 0.f);
        for (int i = 0; i < hei; ++i) {
            const double a = (i < hoi) ? sq(i) / r2 : sq(i), b = (i < hoi) ? 1.0 / (sq(i) * r2) : 1.0 / sq(i);
            for (int j = 0; j < hei; ++j) {
                const double y = Ye[(size_t)i * hei + j];
                AeT[(size_t)i * pe4 + j] = (float)(y * a);  // Ae[j][i]
                BeT[(size_t)j * pe4 + i] = (float)(y * b);  // Be[i][j]
            }
        }
        for (int i = 0; i < hoi; ++i) {
            const double a = sq(i) / r2, b = 1.0 / (sq(i) * r2);
            for (int j = 0; j < hoi; ++j) {
                const double y = Yo[(size_t)i * hoi + j];
                AoT[(size_t)i * po4 + j] = (float)(y * a);
                BoT[(size_t)j * po4 + i] = (float)(y * b);
            }
        }
        // lifting vectors V^T S_I1, V^T S_In: fold M^-1/2 S_I1 orthogonally
        for (int wall = 0; wall < 2; ++wall) {
            const int col = wall ? nz - 1 : 0;
            std::vector<double> gv(ni);
            for (int i = 0; i < ni; ++i) gv[i] = S[(size_t)(i + 1) * nz + col] / sq(i);
            std::vector<float>& dst = wall ? snf : s0f;
            for (int j = 0; j < hei; ++j) {
                double acc = 0.0;
                for (int i = 0; i < hei; ++i) {
                    const double ge = (i < hoi) ? (gv[i] + gv[ni - 1 - i]) / r2 : gv[i];
                    acc += Ye[(size_t)i * hei + j] * ge;
                }
                dst[j] = (float)acc;
            }
            for (int j = 0; j < hoi; ++j) {
                double acc = 0.0;
                for (int i = 0; i < hoi; ++i) acc += Yo[(size_t)i * hoi + j] * (gv[i] - gv[ni - 1 - i]) / r2;
                dst[pe4 + j] = (float)acc;
            }
        }
        for (int j = 0; j < hei; ++j) lamf[j] = (float)le[j];
        for (int j = 0; j < hoi; ++j) lamf[pe4 + j] = (float)lo[j];
        const int nzp = (nz + 3) / 4 * 4;
        std::vector<float> D1e32(D1e.begin(), D1e.end()), D1o32(D1o.begin(), D1o.end());
        auto split = [](const std::vector<double>& a) {
            std::vector<float2> r(a.size());
            for (size_t i = 0; i < a.size(); ++i) {
                r[i].x = (float)a[i];
                r[i].y = (float)(a[i] - (double)r[i].x);
            }
            return r;
        };
        const std::vector<float2> D1e_df = split(D1e), D1o_df = split(D1o), W1e_df = split(W1e), W1o_df = split(W1o);
        std::vector<double> Sfe, Sfo;
        fold_symmetric(S, nz, Sfe, Sfo);
        std::vector<float2> Se_df = split(Sfe), So_df = split(Sfo);
        if (So_df.empty()) So_df.assign(1, float2{0.f, 0.f});
        // eigenbasis of the full Neumann problem S V' = M V' Lambda':
        // C = M^-1/2 S M^-1/2 is centro-symmetric; the orthogonal fold
        // e_i = (x_i + x_{n-1-i})/sqrt2, o_i = (x_i - x_{n-1-i})/sqrt2 (middle
        // kept) splits it into Cne (he x he) and Cno (ho x ho)
        const int he = nz - nz / 2, ho = nz / 2;
        auto Cn = [&](int i, int j) { return S[(size_t)i * nz + j] / std::sqrt(wh[i] * wh[j]); };
        std::vector<double> Cne((size_t)he * he), Cno((size_t)std::max(ho, 1) * std::max(ho, 1), 0.0);
        for (int i = 0; i < he; ++i)
            for (int j = 0; j < he; ++j) {
                double v;
                if (i < ho && j < ho) v = Cn(i, j) + Cn(i, nz - 1 - j);
                else if (i < ho) v = r2 * Cn(i, ho);  // middle column
                else if (j < ho) v = r2 * Cn(ho, j);  // middle row
                else v = Cn(ho, ho);
                Cne[(size_t)i * he + j] = v;
            }
        for (int i = 0; i < ho; ++i)
            for (int j = 0; j < ho; ++j) Cno[(size_t)i * ho + j] = Cn(i, j) - Cn(i, nz - 1 - j);
        std::vector<double> lne, lno, Yne, Yno;
        jacobi_eigen(he, Cne, lne, Yne);
        if (ho > 0) jacobi_eigen(ho, Cno, lno, Yno);
        const int phe4 = (he + 3) / 4 * 4, pho4 = (ho + 3) / 4 * 4;
        // v = M^-1/2 Q y: folded weight of row i of an even / odd eigenvector
        auto fe = [&](int i) { return i < ho ? 1.0 / (r2 * std::sqrt(wh[i])) : 1.0 / std::sqrt(wh[i]); };
        auto fo = [&](int i) { return 1.0 / (r2 * std::sqrt(wh[i])); };
        std::vector<float> PAe((size_t)he * phe4, 0.f), PBe((size_t)he * phe4, 0.f), PAo((size_t)std::max(ho, 1) * pho4 + 4, 0.f),
            PBo((size_t)std::max(ho, 1) * pho4 + 4, 0.f), PDe((size_t)std::max(ho, 1) * phe4 + 4, 0.f),
            PDo((size_t)he * pho4 + 4, 0.f), plame(phe4, 1.f), plamo(pho4 + 4, 1.f);
        for (int i = 0; i < he; ++i)
            for (int j = 0; j < he; ++j) {
                const double a = Yne[(size_t)i * he + j] * fe(i);
                PAe[(size_t)i * phe4 + j] = (float)a;  // forward: out j, sum over i
                PBe[(size_t)j * phe4 + i] = (float)a;  // back: out i, sum over j
            }
        for (int i = 0; i < ho; ++i)
            for (int j = 0; j < ho; ++j) {
                const double a = Yno[(size_t)i * ho + j] * fo(i);
                PAo[(size_t)i * pho4 + j] = (float)a;
                PBo[(size_t)j * pho4 + i] = (float)a;
            }
        // D v for each eigenvector, in FP64 before the one rounding to FP32:
        // even v -> odd D v (values at i < ho), odd v -> even D v (i < he)
        {
            std::vector<double> v(nz), dv(nz);
            for (int j = 0; j < he; ++j) {
                for (int i = 0; i < he; ++i) v[i] = Yne[(size_t)i * he + j] * fe(i);
                for (int i = 0; i < ho; ++i) v[nz - 1 - i] = v[i];
                for (int z = 0; z < nz; ++z) {
                    double a = 0.0;
                    for (int q = 0; q < nz; ++q) a += D1s[(size_t)z * nz + q] * v[q];
                    dv[z] = a;
                }
                for (int i = 0; i < ho; ++i) PDo[(size_t)j * pho4 + i] = (float)dv[i];
            }
            for (int j = 0; j < ho; ++j) {
                std::fill(v.begin(), v.end(), 0.0);
                for (int i = 0; i < ho; ++i) {
                    v[i] = Yno[(size_t)i * ho + j] * fo(i);
                    v[nz - 1 - i] = -v[i];
                }
                for (int z = 0; z < nz; ++z) {
                    double a = 0.0;
                    for (int q = 0; q < nz; ++q) a += D1s[(size_t)z * nz + q] * v[q];
                    dv[z] = a;
                }
                for (int i = 0; i < he; ++i) PDe[(size_t)j * phe4 + i] = (float)dv[i];
            }
        }
        // the same forward operators with input row i scaled by 2 w_i / dt
        std::vector<float> PAeS(PAe.size(), 0.f), PAoS(PAo.size(), 0.f);
        for (int i = 0; i < he; ++i)
            for (int j = 0; j < he; ++j)
                PAeS[(size_t)i * phe4 + j] = (float)(Yne[(size_t)i * he + j] * fe(i) * 2.0 * wh[i] / c.dt);
        for (int i = 0; i < ho; ++i)
            for (int j = 0; j < ho; ++j)
                PAoS[(size_t)i * pho4 + j] = (float)(Yno[(size_t)i * ho + j] * fo(i) * 2.0 * wh[i] / c.dt);
        for (int j = 0; j < he; ++j) plame[j] = (float)lne[j];
        for (int j = 0; j < ho; ++j) plamo[j] = (float)lno[j];
        MixedOps& mx = h->mx;
        mx.nzp = nzp;
        mx.phe4 = phe4;
        mx.pho4 = pho4;
        mx.hei = hei;
        mx.hoi = hoi;
        mx.pe4 = pe4;
        mx.po4 = po4;
        if ((rc = dev_alloc(h, &mx.AeT, AeT.size())) || (rc = dev_alloc(h, &mx.AoT, std::max<size_t>(AoT.size(), 4))) ||
            (rc = dev_alloc(h, &mx.BeT, BeT.size())) || (rc = dev_alloc(h, &mx.BoT, std::max<size_t>(BoT.size(), 4))) ||
            (rc = dev_alloc(h, &mx.lam, lamf.size())) || (rc = dev_alloc(h, &mx.s0, s0f.size())) ||
            (rc = dev_alloc(h, &mx.sn, snf.size())) ||
            (rc = dev_alloc(h, &mx.D1e, D1e32.size())) || (rc = dev_alloc(h, &mx.D1o, D1o32.size())) ||
            (rc = dev_alloc(h, &mx.PAe, PAe.size())) || (rc = dev_alloc(h, &mx.PAo, PAo.size())) ||
            (rc = dev_alloc(h, &mx.PAeS, PAeS.size())) || (rc = dev_alloc(h, &mx.PAoS, PAoS.size())) ||
            (rc = dev_alloc(h, &mx.PBe, PBe.size())) || (rc = dev_alloc(h, &mx.PBo, PBo.size())) ||
            (rc = dev_alloc(h, &mx.PDe, PDe.size())) || (rc = dev_alloc(h, &mx.PDo, PDo.size())) ||
            (rc = dev_alloc(h, &mx.plame, plame.size())) || (rc = dev_alloc(h, &mx.plamo, plamo.size())) ||
            (rc = dev_alloc(h, &mx.D1e_df, D1e_df.size())) || (rc = dev_alloc(h, &mx.D1o_df, D1o_df.size())) ||
            (rc = dev_alloc(h, &mx.W1e_df, W1e_df.size())) || (rc = dev_alloc(h, &mx.W1o_df, W1o_df.size())) ||
            (rc = dev_alloc(h, &mx.Se_df, Se_df.size())) || (rc = dev_alloc(h, &mx.So_df, So_df.size())) ||
            (rc = dev_alloc(h, &h->PHIZ, se)))
            return fail(rc);
        struct Up32 { void* d; const void* s; size_t b; } u32[] = {
            {mx.AeT, AeT.data(), AeT.size() * 4}, {mx.AoT, AoT.data(), AoT.size() * 4},
            {mx.BeT, BeT.data(), BeT.size() * 4}, {mx.BoT, BoT.data(), BoT.size() * 4},
            {mx.lam, lamf.data(), lamf.size() * 4}, {mx.s0, s0f.data(), s0f.size() * 4},
            {mx.sn, snf.data(), snf.size() * 4}, {mx.D1e, D1e32.data(), D1e32.size() * 4},
            {mx.D1o, D1o32.data(), D1o32.size() * 4},
            {mx.PAe, PAe.data(), PAe.size() * 4}, {mx.PAo, PAo.data(), PAo.size() * 4},
            {mx.PAeS, PAeS.data(), PAeS.size() * 4}, {mx.PAoS, PAoS.data(), PAoS.size() * 4},
            {mx.PBe, PBe.data(), PBe.size() * 4}, {mx.PBo, PBo.data(), PBo.size() * 4},
            {mx.PDe, PDe.data(), PDe.size() * 4}, {mx.PDo, PDo.data(), PDo.size() * 4},
            {mx.plame, plame.data(), plame.size() * 4}, {mx.plamo, plamo.data(), plamo.size() * 4},
            {mx.D1e_df, D1e_df.data(), D1e_df.size() * 8}, {mx.D1o_df, D1o_df.data(), D1o_df.size() * 8},
            {mx.W1e_df, W1e_df.data(), W1e_df.size() * 8}, {mx.W1o_df, W1o_df.data(), W1o_df.size() * 8},
            {mx.Se_df, Se_df.data(), Se_df.size() * 8}, {mx.So_df, So_df.data(), So_df.size() * 8}};
        for (auto& u : u32)
            if ((rc = upload(h, u.d, u.s, u.b))) return fail(rc);
        for (int f = 0; f < 6; ++f)
            if ((rc = dev_alloc(h, &h->spec32[f], se)) || (rc = dev_alloc(h, &h->phys32[f], pe))) return fail(rc);
        for (int f = 0; f < 3; ++f)
            if ((rc = dev_alloc(h, &h->src32[f], se))) return fail(rc);
        if ((rc = dev_alloc(h, &h->fft.tmp32, 6 * se))) return fail(rc);
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(DNS3D_E_CUDA);
    }

    // step parameters
    StepParams& sp = h->sp;
    sp.dt = c.dt;
    sp.inv_dt = 1.0 / c.dt;
    sp.cn_fac = c.use_crank_nicolson ? 0.5 * c.dt / c.re : 0.0;
    sp.helm_f = helm_f;
    sp.cn_identity = (sp.cn_fac != 0.0 && sp.cn_fac == helm_f) ? 1 : 0;
    sp.refine = (h->mixed && c.poisson_refinement) ? 1 : 0;
    sp.forcing_scale = (double)c.nx * (double)c.ny;
    sp.dealias = c.use_dealias_23_rule;
    sp.kx_max = (c.nx / 2) * 2 / 3;
    sp.ky_max = (c.ny / 2) * 2 / 3;
    sp.weak_form = c.use_weak_form_divergence;
    PIParams& pp = h->pp;
    pp.method = c.flow_control_method;
    pp.istart = c.istart;
    pp.update_freq = c.controller_update_freq > 0 ? c.controller_update_freq : 1;
    pp.target_dpdx = c.target_pressure_gradient;
    pp.target_ub = c.target_bulk_velocity;
    pp.gain = c.controller_gain;
    pp.re = c.re;
    pp.dt = c.dt;
    double wsum = 0.0;
    for (int k = 0; k < nz; ++k) wsum += h->zwts[k];
    pp.inv_nxny_wsum = 1.0 / ((double)c.nx * (double)c.ny * wsum);

    // tensor-core form of the Helmholtz inverses: FP64 Crank-Nicolson runs with
    // the direct solver (DNS3D_TENSOR_CORES=0 keeps the FP64-pipe kernel)
    if ((rc = dev_alloc(h, &h->d_tcerr, 2))) return fail(rc);
    const char* zcenv = std::getenv("DNS3D_ZERO_COPY");
    h->zero_copy = !(zcenv && std::strcmp(zcenv, "0") == 0);
    const char* tcenv = std::getenv("DNS3D_TENSOR_CORES");
    const char* stall = std::getenv("DNS3D_TC_TEST_STALL");
    ops.tc_stall = stall && std::strcmp(stall, "1") == 0;
    if (!h->mixed && sp.cn_identity && c.linear_solver == 0 && !(tcenv && std::strcmp(tcenv, "0") == 0) &&
        viscous_tc_fits(g)) {
        const TcGeom t = tc_geom(nz);
        __half* sl = nullptr;
        int* ex = nullptr;
        double* tau = nullptr;
        if ((rc = dev_alloc(h, &sl, (size_t)nq * tc_q_halves(t))) || (rc = dev_alloc(h, &ex, (size_t)nq * t.m8)) ||
            (rc = dev_alloc(h, &tau, (size_t)2 * t.he)))
            return fail(rc);
        std::vector<double> th((size_t)2 * t.he, 0.0);
        for (int k = 1; k < t.he; ++k) {
            const double w2 = 2.0 * wh[k];
            if (k < t.ho) {
                th[k] = (S0[k] + Sn[k]) / w2;
                th[t.he + k] = (S0[k] - Sn[k]) / w2;
            } else {
                th[k] = S0[k] / w2;  // the unpaired mid level (S0 = Sn there)
            }
        }
        if ((rc = upload(h, tau, th.data(), th.size() * sizeof(double)))) return fail(rc);
        if ((e = build_tc_slices(g, ops.HinvF, ops.wh, nq, sl, ex, h->stream)) ||
            (e = cudaStreamSynchronize(h->stream))) {
            cuda_fail(h, e, "build_tc_slices");
            return fail(DNS3D_E_CUDA);
        }
        ops.tcA = sl;
        ops.tcE = ex;
        ops.tcTau = tau;
        h->visc_tc_forced = tcenv && std::strcmp(tcenv, "1") == 0;
        // without timing: the tensor-core kernel once the grid has a few waves
        // of operator pairs and two of its CTAs fit an SM
        h->visc_tc = h->visc_tc_forced || (nq >= 8 * 152 && viscous_tc_smem(g) <= 113 * 1024);
    }
    // the folded D1 as a digit image for the tensor-core vorticity (FP64 runs)
    if (!h->mixed && !(tcenv && std::strcmp(tcenv, "0") == 0) && vorticity_tc_fits(g)) {
        const TcGeom t = tc_geom(nz);
        __half* im = nullptr;
        int* ex = nullptr;
        if ((rc = dev_alloc(h, &im, (size_t)kTcSlices * tc_blocks(t, true).a)) || (rc = dev_alloc(h, &ex, (size_t)t.m8)))
            return fail(rc);
        if ((e = build_tc_anti_image(g, ops.D1e, ops.D1o, im, ex, h->stream)) ||
            (e = cudaStreamSynchronize(h->stream))) {
            cuda_fail(h, e, "build_tc_anti_image");
            return fail(DNS3D_E_CUDA);
        }
        ops.tcD = im;
        ops.tcDE = ex;
        // the Poisson inverses in fixed point for the solve after the
        // tensor-core right-hand side (the strong form)
        if (!c.use_weak_form_divergence) {
            const size_t qs = fx_qstride(ops.he, ops.ho);
            long long* gi = nullptr;
            int* ge = nullptr;
            if ((rc = dev_alloc(h, &gi, (size_t)nq * qs)) || (rc = dev_alloc(h, &ge, (size_t)nq * nz)))
                return fail(rc);
            if ((e = build_fixed_rows(g, ops.PinvF, nq, gi, ge, h->stream)) || (e = cudaStreamSynchronize(h->stream))) {
                cuda_fail(h, e, "build_fixed_rows");
                return fail(DNS3D_E_CUDA);
            }
            ops.PinvI = gi;
            ops.PinvE = ge;
        }
        h->visc_tc_forced = tcenv && std::strcmp(tcenv, "1") == 0;
        h->vort_tc = h->visc_tc_forced || g.nm >= 4 * 152 * 8;
        h->corr_tc = h->visc_tc_forced || g.nm >= 4 * 152 * 16;
        h->pres_tc = ops.PinvI && (h->visc_tc_forced || g.nm >= 4 * 152 * 16);
    }

    if ((rc = dns3d_initialize_fields(h))) return fail(rc);
    const char* at = std::getenv("DNS3D_AUTOTUNE");
    if (!(at && std::strcmp(at, "0") == 0))
        if ((rc = autotune(h, false))) return fail(rc);
    *out = h;
    return DNS3D_OK;
}

int dns3d_destroy(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    cudaSetDevice(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    release(h);
    delete h;
    return DNS3D_OK;
}

}  // extern "C"

namespace {

// generate_channel_solenoidal_perturbations (perturbation_module.f90:42-176)
// with a seeded stream in place of the clock-seeded random_number: random
// spectra of u and v (four draws per mode, k, j, i order), high-wavenumber
// damping, per-mode projection onto kx u + ky v = 0 (real and imaginary
// parts separately), zero mean mode; c2r to physical space; w from the
// trapezoid integration of -(du/dx + dv/dy) (or zero); walls zeroed and the
// interior damped by (1 - z^2)^2; scaled to mean energy amplitude * 0.5 * 1.5^2.
// The transforms and the x-y divergence run on the device.
int random_perturbation(dns3d_handle* h, std::vector<double>& up, std::vector<double>& vp, std::vector<double>& wp) {
    const dns3d_config& c = h->cfg;
    const GridDev& g = h->g;
    const int nx = c.nx, ny = c.ny, nz = c.nz, nxhp = nx / 2 + 1;
    const double pi = 4.0 * std::atan(1.0);
    const size_t ns = (size_t)nz * ny * nxhp, pl = (size_t)nx * ny, N = pl * nz;
    std::vector<double2> uh(ns), vh(ns);
    SplitMix64 rng{(uint64_t)c.perturbation_seed};
    for (size_t o = 0; o < ns; ++o) {
        uh[o].x = rng.uniform() - 0.5;
        uh[o].y = rng.uniform() - 0.5;
        vh[o].x = rng.uniform() - 0.5;
        vh[o].y = rng.uniform() - 0.5;
    }
    const double kcut = 0.5 * std::min(2.0 * pi * nx / c.xlen, 2.0 * pi * ny / c.ylen);
    for (int k = 0; k < nz; ++k)
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nxhp; ++i) {
                double2& a = uh[((size_t)k * ny + (j - 1)) * nxhp + (i - 1)];
                double2& b = vh[((size_t)k * ny + (j - 1)) * nxhp + (i - 1)];
                const double kx = 2.0 * pi * (double)(i - 1) / c.xlen;
                const double ky = 2.0 * pi * (double)(j <= ny / 2 + 1 ? j - 1 : j - 1 - ny) / c.ylen;
                const double kp = kx * kx + ky * ky;
                if (std::sqrt(kp) > kcut) {
                    a.x *= 0.1; a.y *= 0.1;
                    b.x *= 0.1; b.y *= 0.1;
                }
                if (kp > 1.0e-12) {
                    double kv = kx * a.x + ky * b.x;
                    a.x -= kx * kv / kp;
                    b.x -= ky * kv / kp;
                    kv = kx * a.y + ky * b.y;
                    a.y -= kx * kv / kp;
                    b.y -= ky * kv / kp;
                }
                if (i == 1 && j == 1) a = b = make_double2(0.0, 0.0);
            }
    const size_t sb = ns * sizeof(double2), pb = N * sizeof(double);
    CK(h, cudaMemcpyAsync(h->U, uh.data(), sb, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->V, vh.data(), sb, cudaMemcpyHostToDevice, h->stream));
    Fields sp{};
    sp.p[0] = h->U; sp.p[1] = h->V;
    RFields ph{};
    ph.p[0] = h->phys[0]; ph.p[1] = h->phys[1];
    CK(h, fft_c2r(h->fft, g, sp, ph, 2, nz, h->stream));
    up.resize(N);
    vp.resize(N);
    wp.assign(N, 0.0);
    CK(h, cudaMemcpyAsync(up.data(), h->phys[0], pb, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(vp.data(), h->phys[1], pb, cudaMemcpyDeviceToHost, h->stream));
    if (!c.zero_w_perturbations) {
        // compute_spectral_derivatives_xy: du/dx + dv/dy of the physical fields
        CK(h, fft_r2c(h->fft, g, ph, sp, 2, nz, h->stream));
        CK(h, cudaMemsetAsync(h->W, 0, sb, h->stream));
        double2* div = h->fft.tmp + (size_t)5 * spec_elems(c);
        CK(h, launch_divergence(g, h->ops, h->U, h->V, h->W, div, h->stream));
        Fields dv{}; dv.p[0] = div;
        RFields dp{}; dp.p[0] = h->phys[2];
        CK(h, fft_c2r(h->fft, g, dv, dp, 1, nz, h->stream));
        std::vector<double> dxy(N);
        CK(h, cudaMemcpyAsync(dxy.data(), h->phys[2], pb, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        std::vector<double> col(nz), wc(nz);
        for (size_t p = 0; p < pl; ++p) {
            for (int k = 0; k < nz; ++k) col[k] = dxy[k * pl + p];
            integrate_w_column(nz, h->zpts.data(), col.data(), wc.data());
            for (int k = 0; k < nz; ++k) wp[k * pl + p] = wc[k];
        }
    }
    CK(h, cudaStreamSynchronize(h->stream));
    h->phys_valid = 0;
    // enforce_channel_walls (perturbation_module.f90:276-320)
    for (int k = 0; k < nz; ++k) {
        const double d = (k == 0 || k == nz - 1) ? 0.0 : (1.0 - h->zpts[k] * h->zpts[k]) * (1.0 - h->zpts[k] * h->zpts[k]);
        for (size_t p = 0; p < pl; ++p) {
            up[k * pl + p] *= d;
            vp[k * pl + p] *= d;
            wp[k * pl + p] *= d;
        }
    }
    // scale_to_amplitude (perturbation_module.f90:325-372)
    double su = 0.0, sv = 0.0, sw = 0.0;
    for (size_t o = 0; o < N; ++o) { su += up[o] * up[o]; sv += vp[o] * vp[o]; sw += wp[o] * wp[o]; }
    const double cur = 0.5 * (su + sv + sw) / (double)N;
    const double target = c.perturbation_amplitude * (0.5 * 1.5 * 1.5);
    const double sc = cur > 1.0e-15 ? std::sqrt(target / cur) : 1.0;
    for (size_t o = 0; o < N; ++o) { up[o] *= sc; vp[o] *= sc; wp[o] *= sc; }
    return DNS3D_OK;
}

}  // namespace

extern "C" {

int dns3d_initialize_fields(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    std::vector<double> u, v, w;
    initial_fields(h->cfg, h->zpts, u, v, w);
    if (h->cfg.enable_perturbations && !h->cfg.use_analytical_perturbations) {
        // apply_solenoidal_perturbations (3D:3219-3259): add, then the walls again
        std::vector<double> up, vp, wp;
        const int rp = random_perturbation(h, up, vp, wp);
        if (rp) return rp;
        const size_t pl = (size_t)h->cfg.nx * h->cfg.ny;
        for (size_t o = 0; o < u.size(); ++o) { u[o] += up[o]; v[o] += vp[o]; w[o] += wp[o]; }
        for (int k : {0, h->cfg.nz - 1})
            for (size_t i = 0; i < pl; ++i) { u[k * pl + i] = 0.0; v[k * pl + i] = 0.0; w[k * pl + i] = 0.0; }
    }
    if (h->cfg.noise_amplitude > 0.0) {
        const uint64_t seed = (uint64_t)h->cfg.perturbation_seed;
        const double a = h->cfg.noise_amplitude;
        double* f[3] = {u.data(), v.data(), w.data()};
        const size_t n = u.size();
        const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
                for (int comp = 0; comp < 3; ++comp)
                    for (size_t o = lo; o < hi; ++o) f[comp][o] += noise_sample(seed, o, comp, a);
            });
        for (auto& th : pool) th.join();
        const size_t pl = (size_t)h->cfg.nx * h->cfg.ny;
        for (int k : {0, h->cfg.nz - 1})
            for (size_t i = 0; i < pl; ++i) { u[k * pl + i] = 0.0; v[k * pl + i] = 0.0; w[k * pl + i] = 0.0; }
    }
    std::vector<double> p(u.size(), 0.0);
    const size_t pl = (size_t)h->cfg.nx * h->cfg.ny;
    std::vector<double> zero(pl, 0.0);
    dns3d_pi_state pi{};
    pi.current_pressure_gradient = h->cfg.target_pressure_gradient;  // 3D:623
    pi.avg_pressure_gradient = h->cfg.target_pressure_gradient;      // 3D:635
    int rc = dns3d_set_state(h, u.data(), v.data(), w.data(), p.data(), zero.data(), zero.data(),
                             zero.data(), zero.data(), &pi);
    if (rc) return rc;
    h->step = 0;
    h->time = 0.0;
    return DNS3D_OK;
}

int dns3d_set_state(dns3d_handle* h, const double* u, const double* v, const double* w,
                    const double* p_total, const double* gpx_w1, const double* gpx_w2,
                    const double* gpy_w1, const double* gpy_w2, const dns3d_pi_state* pi) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    const GridDev& g = h->g;
    const size_t pe = phys_elems(h->cfg);
    const double* src[4] = {u, v, w, p_total};
    double2* dst[4] = {h->U, h->V, h->W, h->P};
    int rc;
    h->phys_valid = 0;
    // Two batches: the first half of the given fields is uploaded on the
    // handle's stream and transformed there while the second half is still
    // being copied on the side stream; the second batch's transform waits
    // for its copies.
    int idx[4], n = 0;
    for (int f = 0; f < 4; ++f)
        if (src[f]) idx[n++] = f;
    // pinned buffers: the x pass of the transform reads them in place
    bool in_place = h->zero_copy && n > 0;
    RFields hv{};
    for (int i = 0; i < n && in_place; ++i) {
        hv.p[i] = device_view(src[idx[i]]);
        in_place = hv.p[i] != nullptr;
    }
    if (in_place) {
        Fields sp{};
        for (int i = 0; i < n; ++i) sp.p[i] = dst[idx[i]];
        CK(h, fft_r2c(h->fft, g, hv, sp, n, g.nz, h->stream, 0, true));
        n = 0;  // nothing left for the copies below
    }
    const int na = (n + 1) / 2;
    if (n > na) CK(h, fork_side(h, 0));  // the side copies wait for prior work on phys[]
    for (int i = 0; i < n; ++i) {
        const int f = idx[i];
        CK(h, cudaMemcpyAsync(h->phys[f], src[f], pe * sizeof(double), cudaMemcpyHostToDevice,
                              i < na ? h->stream : side_stream(h)));
    }
    for (int b = 0; b < 2; ++b) {
        const int lo = b ? na : 0, hi = b ? n : na;
        if (lo == hi) continue;
        if (b) CK(h, join_side(h, 0));
        RFields ph{};
        Fields sp{};
        for (int i = lo; i < hi; ++i) {
            ph.p[i - lo] = h->phys[idx[i]];
            sp.p[i - lo] = dst[idx[i]];
        }
        CK(h, fft_r2c(h->fft, g, ph, sp, hi - lo, g.nz, h->stream));
    }
    const double* gps[4] = {gpx_w1, gpx_w2, gpy_w1, gpy_w2};
    const bool any_gp = gpx_w1 || gpx_w2 || gpy_w1 || gpy_w2;
    const size_t pl = (size_t)g.nx * g.ny;
    if (any_gp) {
        for (int i = 0; i < 4; ++i) {
            if (!gps[i]) continue;
            if ((rc = upload(h, h->phys[4], gps[i], pl * sizeof(double)))) return rc;
            RFields ph{}; ph.p[0] = h->phys[4];
            Fields sp{}; sp.p[0] = h->GP + (size_t)i * g.nm;
            CK(h, fft_r2c(h->fft, g, ph, sp, 1, 1, h->stream));
        }
    } else if (p_total) {
        CK(h, launch_grad_walls(g, h->ops, h->P, h->GP, h->stream));
    }
    if (pi) {
        if ((rc = upload(h, h->d_pi, pi, sizeof(*pi)))) return rc;
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return DNS3D_OK;
}

int dns3d_get_state(dns3d_handle* h, double* u, double* v, double* w, double* p_total,
                    double* gpx_w1, double* gpx_w2, double* gpy_w1, double* gpy_w2,
                    dns3d_pi_state* pi) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    const GridDev& g = h->g;
    const size_t pe = phys_elems(h->cfg);
    double* dst[4] = {u, v, w, p_total};
    double2* src[4] = {h->U, h->V, h->W, h->P};
    // Requested fields already in phys[] are copied at once on the side
    // stream; the others are transformed in two batches, the first batch's
    // copies (side stream) overlapping the second batch's transform.
    int need[4], n = 0, have[4], nh = 0;
    for (int f = 0; f < 4; ++f) {
        if (!dst[f]) continue;
        if (h->phys_valid >> f & 1u) have[nh++] = f;
        else need[n++] = f;
    }
    // pinned buffers and fixed-point transforms: the x pass writes each field
    // to phys[] (kept for the diagnostics) and to the host buffer in one pass
    bool in_place = h->zero_copy && h->fft.fx && n > 0;
    RFields hv{};
    for (int i = 0; i < n && in_place; ++i) {
        hv.p[i] = device_view(dst[need[i]]);
        in_place = hv.p[i] != nullptr;
    }
    if (in_place) {
        Fields sp{};
        RFields ph{};
        for (int i = 0; i < n; ++i) {
            sp.p[i] = src[need[i]];
            ph.p[i] = h->phys[need[i]];
        }
        CK(h, fft_c2r_copy(h->fft, g, sp, ph, hv, n, g.nz, h->stream));
        for (int i = 0; i < n; ++i) h->phys_valid |= 1u << need[i];
        n = 0;
    }
    const int na = (n + 1) / 2;
    const bool side = nh > 0 || n > 1;
    if (side) CK(h, fork_side(h, 0));
    for (int i = 0; i < nh; ++i)
        CK(h, cudaMemcpyAsync(dst[have[i]], h->phys[have[i]], pe * sizeof(double), cudaMemcpyDeviceToHost,
                              side_stream(h)));
    for (int b = 0; b < 2; ++b) {
        const int lo = b ? na : 0, hi = b ? n : na;
        if (lo == hi) continue;
        Fields sp{};
        RFields ph{};
        for (int i = lo; i < hi; ++i) {
            sp.p[i - lo] = src[need[i]];
            ph.p[i - lo] = h->phys[need[i]];
        }
        CK(h, fft_c2r(h->fft, g, sp, ph, hi - lo, g.nz, h->stream));
        if (b == 0 && n > 1) CK(h, fork_side(h, 1));  // the side stream copies batch 0 after its transform
        for (int i = lo; i < hi; ++i)
            CK(h, cudaMemcpyAsync(dst[need[i]], h->phys[need[i]], pe * sizeof(double), cudaMemcpyDeviceToHost,
                                  (b == 0 && n > 1) ? side_stream(h) : h->stream));
    }
    if (side) CK(h, join_side(h, 0));
    for (int f = 0; f < 4; ++f)
        if (dst[f]) h->phys_valid |= 1u << f;
    double* gps[4] = {gpx_w1, gpx_w2, gpy_w1, gpy_w2};
    const size_t pl = (size_t)g.nx * g.ny;
    for (int i = 0; i < 4; ++i) {
        if (!gps[i]) continue;
        Fields gsp{}; gsp.p[0] = h->GP + (size_t)i * g.nm;
        RFields gph{}; gph.p[0] = h->phys[4];
        CK(h, fft_c2r(h->fft, g, gsp, gph, 1, 1, h->stream));
        CK(h, cudaMemcpyAsync(gps[i], h->phys[4], pl * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    if (pi) CK(h, cudaMemcpyAsync(pi, h->d_pi, sizeof(*pi), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return DNS3D_OK;
}

int dns3d_get_config(dns3d_handle* h, dns3d_config* cfg) {
    if (!h || !cfg) return DNS3D_E_INVALID;
    *cfg = h->cfg;
    return DNS3D_OK;
}

int dns3d_set_clock(dns3d_handle* h, int step, double time) {
    if (!h) return DNS3D_E_INVALID;
    h->step = step;
    h->time = time;
    return DNS3D_OK;
}

int dns3d_compute_source_terms(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    return run_source_terms(h);
}
int dns3d_viscous_step(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    return run_viscous(h);
}
int dns3d_solve_pressure(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    return run_pressure(h);
}
int dns3d_pressure_correction(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    return run_correction(h);
}
int dns3d_apply_boundary_conditions(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    return run_bc(h);
}

int dns3d_step(dns3d_handle* h, int nsteps) {
    if (!h || nsteps < 0) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    if (nsteps == 0) return DNS3D_OK;
    if (!h->graph) {
        cudaGraph_t graph = nullptr;
        CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = run_step_body(h);
        cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&h->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            h->graph = nullptr;
            return cuda_fail(h, e, "cudaGraphInstantiate");
        }
    }
    h->phys_valid = 0;
    for (int s = 0; s < nsteps; ++s) {
        CK(h, cudaGraphLaunch(h->graph, h->stream));
        h->step += 1;
        h->time += h->cfg.dt;  // 3D:296
    }
    return DNS3D_OK;
}

int dns3d_step_timed(dns3d_handle* h, int nsteps, double* elapsed_ms) {
    if (!h || !elapsed_ms || nsteps < 1) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    if (!h->graph) {  // capture outside the timed region
        int rc = dns3d_step(h, 1);
        if (rc) return rc;
    }
    cudaEvent_t e0, e1;
    CK(h, cudaEventCreate(&e0));
    CK(h, cudaEventCreate(&e1));
    CK(h, cudaEventRecord(e0, h->stream));
    int rc = dns3d_step(h, nsteps);
    CK(h, cudaEventRecord(e1, h->stream));
    CK(h, cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(h, cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *elapsed_ms = ms;
    return rc;
}

int dns3d_profile_kernels(dns3d_handle* h, int nsteps, dns3d_kernel_time* out, int cap, int* n) {
    if (!h || !out || !n || cap < 1 || nsteps < 1) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    std::vector<dns3d_kernel_time> acc;
    for (int s = 0; s < nsteps; ++s) {
        h->prof = true;
        h->nev = 0;
        mark(h, "start");
        int rc = run_step_body(h);
        h->prof = false;
        if (rc) return rc;
        CK(h, cudaStreamSynchronize(h->stream));
        h->step += 1;
        h->time += h->cfg.dt;
        for (size_t i = 1; i < h->nev; ++i) {
            float ms = 0.f;
            CK(h, cudaEventElapsedTime(&ms, h->ev[i - 1], h->ev[i]));
            const char* nm = h->evname[i];
            size_t j = 0;
            while (j < acc.size() && std::strcmp(acc[j].name, nm) != 0) ++j;
            if (j == acc.size()) acc.push_back(dns3d_kernel_time{nm, 0, 0, 0.0});
            acc[j].launches += 1;
            acc[j].total_ms += ms;
        }
    }
    const int m = (int)acc.size() < cap ? (int)acc.size() : cap;
    for (int i = 0; i < m; ++i) out[i] = acc[i];
    *n = m;
    return DNS3D_OK;
}

int dns3d_launches_per_step(dns3d_handle* h, int* n) {
    if (!h || !n) return DNS3D_E_INVALID;
    if (h->launches == 0) {  // count by a dry capture-free pass is not possible; run one step
        int rc = dns3d_step(h, 1);
        if (rc) return rc;
    }
    *n = h->launches;
    return DNS3D_OK;
}

int dns3d_check_conversions(int device, long long n, unsigned long long* mismatches) {
    if (!mismatches || n < 1) return DNS3D_E_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return DNS3D_E_CUDA;
    return check_conversions(n, mismatches) == cudaSuccess ? DNS3D_OK : DNS3D_E_CUDA;
}

int dns3d_measure_fp64_tflops(int device, double* tflops) {
    if (!tflops) return DNS3D_E_INVALID;
    cudaError_t e = measure_fp64_tflops(device, tflops);
    return e == cudaSuccess ? DNS3D_OK : DNS3D_E_CUDA;
}

int dns3d_synchronize(dns3d_handle* h) {
    if (!h) return DNS3D_E_INVALID;
    CK(h, cudaStreamSynchronize(h->stream));
    return DNS3D_OK;
}

int dns3d_query(dns3d_handle* h, int* done) {
    if (!h || !done) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    const cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaErrorNotReady) {
        // not an error; make sure a later launch check cannot read it as one
        if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
        *done = 0;
        return DNS3D_OK;
    }
    CK(h, e);
    *done = 1;
    return DNS3D_OK;
}

}  // extern "C"

namespace {

// output_diagnostics_3d's reductions (and, with `div`, check_divergence_3d's)
// of the device state; `mean` receives the (0,0) mode of u, v, w per level
// when non-null (3 * nz values, plane sums of the physical fields).
int diag_core(dns3d_handle* h, dns3d_diag* out, bool with_div, std::vector<double2>* mean3) {
    CK(h, cudaSetDevice(h->cfg.device));
    const GridDev& g = h->g;
    const dns3d_config& c = h->cfg;
    // the physical u, v, w: reuse what get_state left in phys[], transform the rest
    const double2* spec[3] = {h->U, h->V, h->W};
    Fields sp{};
    RFields ph{};
    int nf = 0;
    for (int f = 0; f < 3; ++f) {
        if (h->phys_valid >> f & 1u) continue;
        sp.p[nf] = const_cast<double2*>(spec[f]);
        ph.p[nf] = h->phys[f];
        ++nf;
    }
    if (nf) CK(h, fft_c2r(h->fft, g, sp, ph, nf, g.nz, h->stream));
    h->phys_valid |= 7u;
    CK(h, launch_diag_reduce(g, h->ops, h->phys[0], h->phys[1], h->phys[2], h->d_red, h->red_blocks, h->d_out,
                             h->stream));
    if (with_div) {
        // check_divergence_3d: max |DX u + DY v + Dz w| in physical space
        // (the divergence spectrum goes to the last FFT scratch slot, which a
        // one-field c2r does not touch, so diagnostics never clobber step state)
        double2* div = h->fft.tmp + (size_t)5 * spec_elems(c);
        CK(h, launch_divergence(g, h->ops, h->U, h->V, h->W, div, h->stream));
        Fields dv{}; dv.p[0] = div;
        RFields dp{}; dp.p[0] = h->phys[3];
        h->phys_valid &= ~8u;  // phys[3] now holds the divergence
        CK(h, fft_c2r(h->fft, g, dv, dp, 1, g.nz, h->stream));
        CK(h, launch_maxabs(g, h->phys[3], phys_elems(c), h->d_red, h->red_blocks, h->d_out + 4, h->stream));
    }
    // results, controller state and the (0,0) modes in one block, one copy:
    // d_out = [5 reductions, 3 spare][dns3d_pi_state (8 doubles)][3 nz complex]
    constexpr int kPiDoubles = (int)(sizeof(dns3d_pi_state) / sizeof(double));
    CK(h, launch_diag_gather(g, h->U, h->V, h->W, h->d_pi, h->d_out + 8, h->stream));
    CK(h, cudaMemcpyAsync(h->d_out + 5, h->d_tcerr, 2 * sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
    const size_t nblk = 8 + kPiDoubles + 6 * (size_t)g.nz;
    CK(h, cudaMemcpyAsync(h->h_out, h->d_out, nblk * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    const std::vector<double> blk(h->h_out, h->h_out + nblk);
    double res[5] = {blk[0], blk[1], blk[2], blk[3], with_div ? blk[4] : 0.0};
    dns3d_pi_state pi{};
    std::memcpy(&pi, blk.data() + 8, sizeof(pi));
    std::vector<double2> mean_local;
    std::vector<double2>& mean = mean3 ? *mean3 : mean_local;
    mean.resize((size_t)3 * g.nz);
    std::memcpy(mean.data(), blk.data() + 8 + kPiDoubles, mean.size() * sizeof(double2));
    const double ybar = 2.0;
    const double fac = (c.xlen / c.nx) * (c.ylen / c.ny) * (ybar / 2.0);
    out->umax = res[0];
    out->vmax = res[1];
    out->wmax = res[2];
    out->energy = res[3] * fac / (c.xlen * c.ylen * ybar);  // 3D:2110-2128
    out->max_div = res[4];
    out->dpdx = pi.current_pressure_gradient;
    out->dpdx_avg = pi.avg_pressure_gradient;
    double vol = 0.0;
    for (int k = 0; k < g.nz; ++k) vol += mean[k].x * h->zwts[k];
    out->u_bulk = vol * h->pp.inv_nxny_wsum;
    out->time = h->time;
    out->step = h->step;
    long long tcerr = 0;
    std::memcpy(&tcerr, &blk[5], sizeof(tcerr));
    if (tcerr) {
        h->err = "a tensor-core completion wait ran out";
        return DNS3D_E_TIMEOUT;
    }
    if (!std::isfinite(out->energy) || !std::isfinite(out->umax) || !std::isfinite(out->max_div))
        return DNS3D_E_NONFINITE;
    return DNS3D_OK;
}

}  // namespace

extern "C" {

int dns3d_diagnostics(dns3d_handle* h, dns3d_diag* out) {
    if (!h || !out) return DNS3D_E_INVALID;
    return diag_core(h, out, true, nullptr);
}

int dns3d_output_diagnostics(dns3d_handle* h, dns3d_diag* out) {
    if (!h || !out) return DNS3D_E_INVALID;
    return diag_core(h, out, false, nullptr);
}

int dns3d_check_divergence(dns3d_handle* h, double* max_div) {
    if (!h || !max_div) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    const GridDev& g = h->g;
    const dns3d_config& c = h->cfg;
    double2* div = h->fft.tmp + (size_t)5 * spec_elems(c);
    CK(h, launch_divergence(g, h->ops, h->U, h->V, h->W, div, h->stream));
    Fields dv{}; dv.p[0] = div;
    RFields dp{}; dp.p[0] = h->phys[3];
    h->phys_valid &= ~8u;  // phys[3] now holds the divergence
    CK(h, fft_c2r(h->fft, g, dv, dp, 1, g.nz, h->stream));
    CK(h, launch_maxabs(g, h->phys[3], phys_elems(c), h->d_red, h->red_blocks, h->d_out + 4, h->stream));
    CK(h, cudaMemcpyAsync(max_div, h->d_out + 4, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return std::isfinite(*max_div) ? DNS3D_OK : DNS3D_E_NONFINITE;
}

int dns3d_projection_residual(dns3d_handle* h, double* rel) {
    if (!h || !rel) return DNS3D_E_INVALID;
    CK(h, cudaSetDevice(h->cfg.device));
    unsigned long long* buf = reinterpret_cast<unsigned long long*>(h->d_red);
    CK(h, launch_poisson_residual(h->g, h->ops, h->sp, h->US, h->VS, h->WS, h->PHI, buf, h->stream));
    unsigned long long bits[2] = {0, 0};
    CK(h, cudaMemcpyAsync(bits, buf, sizeof(bits), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    double r, b;
    std::memcpy(&r, &bits[0], sizeof(double));
    std::memcpy(&b, &bits[1], sizeof(double));
    *rel = b > 0.0 ? r / b : r;
    return std::isfinite(*rel) ? DNS3D_OK : DNS3D_E_NONFINITE;
}

int dns3d_flow_statistics(dns3d_handle* h, dns3d_flow_stats* out, double* u_avg, double* v_avg, double* w_avg) {
    if (!h || !out) return DNS3D_E_INVALID;
    dns3d_diag d{};
    std::vector<double2> mean;
    const int rc = diag_core(h, &d, false, &mean);
    if (rc && rc != DNS3D_E_NONFINITE) return rc;
    const dns3d_config& c = h->cfg;
    const int nz = c.nz;
    const double nxny = (double)c.nx * (double)c.ny;
    std::memset(out, 0, sizeof(*out));
    out->umax = d.umax;
    out->vmax = d.vmax;
    out->wmax = d.wmax;
    out->energy = d.energy;
    out->dpdx = d.dpdx;
    out->dpdx_avg = d.dpdx_avg;
    out->flow_control_method = c.flow_control_method;
    // bulk velocity: calculate_bulk_velocity_3d for method 2 (3D:2434-2464),
    // sum u*zwts / (nx*ny) / 2 otherwise (3D:2874-2889)
    if (c.flow_control_method == 2) {
        out->bulk_velocity = d.u_bulk;
    } else {
        double vol = 0.0;
        for (int k = 0; k < nz; ++k) vol += mean[k].x * h->zwts[k];
        out->bulk_velocity = vol / nxny / 2.0;
    }
    // wall shear by one-sided differences of the plane means (3D:2891-2921)
    const double nu = 1.0 / c.re;
    const double* z = h->zpts.data();
    const double dl = (mean[1].x - mean[0].x) / nxny / (z[1] - z[0]);
    const double du = (mean[nz - 1].x - mean[nz - 2].x) / nxny / (z[nz - 1] - z[nz - 2]);
    out->wall_shear_lower = nu * dl;
    out->wall_shear_upper = nu * du;
    out->friction_velocity_avg = std::sqrt((std::fabs(out->wall_shear_lower) + std::fabs(out->wall_shear_upper)) / 2.0);
    out->re_tau = out->friction_velocity_avg * c.re;  // 3D:2948-2949
    out->time = h->time;
    out->step = h->step;
    double* dst[3] = {u_avg, v_avg, w_avg};
    for (int f = 0; f < 3; ++f)
        if (dst[f])
            for (int k = 0; k < nz; ++k) dst[f][k] = mean[(size_t)f * nz + k].x / nxny;  // 3D:2819-2833
    return rc;
}

int dns3d_get_clock(dns3d_handle* h, int* step, double* time) {
    if (!h || !step || !time) return DNS3D_E_INVALID;
    *step = h->step;
    *time = h->time;
    return DNS3D_OK;
}

int dns3d_lgl_nodes_weights(int nz, double* z, double* w) {
    if (nz < 3 || !z || !w) return DNS3D_E_INVALID;
    std::vector<double> x, wt;
    lgl_nodes_weights(nz, x, wt);
    for (int k = 0; k < nz; ++k) {
        z[k] = x[k];
        w[k] = wt[k];
    }
    return DNS3D_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batches
// Joint stepping of independent runs.  Eligible runs of one precision and one
// kernel variant (which stages run their tensor-core bodies) form a group
// whose step is ten ragged stage launches (ragged.cuh): a group's launch sizes
// its shared memory for its largest run, so runs of different variants are not
// mixed.  The others keep their own step bodies; every group and loose run is
// a branch of the same graph.
struct dns3d_batch {
    struct Group {
        int key = 0;                  // precision and variant
        bool mixed = false;
        int variant = 0;              // RaggedVariant bits (FP64 groups)
        cudaStream_t lane = nullptr, side = nullptr;  // side: the mixed form's mode (0,0) stages
        cudaEvent_t lane_join = nullptr, side_fork = nullptr, side_join = nullptr;
        std::vector<int> idx;         // runs of the group (indices into runs)
        std::vector<RunDesc> desc;    // host copies of the descriptors
        std::vector<int> own_tc;      // per run, the tile widths of its own launches [kTileKernels]
        RunDesc* d_desc = nullptr;    // [n]
        int* d_map = nullptr;         // per stage: start [n + 1], order [n]
        int total[kRsStages] = {};    // CTAs of each stage launch
        size_t smem[kRsStages] = {};  // dynamic shared memory of each stage launch
    };
    std::vector<dns3d_handle*> runs;  // not owned
    int device = 0;
    cudaStream_t stream = nullptr;    // the batch's graph runs here
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> run_in, run_join;
    std::vector<Group> grp;
    std::vector<int> loose;           // runs stepped by their own launches
    cudaGraphExec_t graph = nullptr;
    int launches = 0;                 // kernel launches per step
    std::string err;
};

namespace {

size_t stage_smem_limit(StageKernel k) {
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, (const void*)k) != cudaSuccess)
        return 0;
    return (size_t)optin - fa.sharedSizeBytes;
}

// Raises every stage kernel's dynamic shared-memory limit to the device's
// opt-in maximum (a property of the kernel, shared by all batches).
cudaError_t prepare_stage_kernels() {
    for (int m = 0; m < 2 * 32; ++m)  // precision x RaggedVariant bits
        for (int s = 0; s < kRsStages; ++s) {
            StageKernel k = ragged_kernel(s, m & 1, m >> 1);
            const size_t lim = stage_smem_limit(k);
            if (!lim) return cudaErrorInvalidValue;
            cudaError_t e = cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim);
            if (e) return e;
        }
    return cudaSuccess;
}

// Runs of 2^20 points and more keep their own launches: they fill the GPU by
// themselves, and their own kernels read every operand from the constant bank
// where the stage bodies hold descriptor fields in registers (one 256x256x97
// mixed run: 1.28 ms per step alone, 1.34 ms as a batch of one).
constexpr long long kRaggedMaxPoints = 1LL << 20;

bool ragged_eligible(const dns3d_handle* h) {
    const long long points = (long long)h->cfg.nx * h->cfg.ny * h->cfg.nz;
    // (a mixed run with the Poisson refinement keeps its own launches: its
    // pressure body is a separate kernel instantiation)
    return h->fft.use_ct && h->cfg.convection_scheme == 0 && h->cfg.linear_solver == 0 && !h->sp.refine &&
           points < kRaggedMaxPoints;
}

RunDesc make_desc(const dns3d_handle* h) {
    RunDesc d{};
    d.g = h->g;
    for (int k = 0; k < kTileKernels; ++k) d.g.tc[k] = tile_width(h->g, k);
    d.ops = h->ops;
    if (!h->visc_tc) {
        d.ops.tcA = nullptr;
        d.ops.tcE = nullptr;
    }
    d.tcmask = (h->vort_tc ? 1 : 0) | (h->corr_tc ? 2 : 0) | (h->pres_tc ? 4 : 0);
    if (!d.tcmask) {
        d.ops.tcD = nullptr;
        d.ops.tcDE = nullptr;
    }
    d.mx = h->mx;
    d.sp = h->sp;
    d.sp.bc_walls = 1;  // batches take whole steps: the projection stage writes the wall planes
    d.pp = h->pp;
    d.pi = h->d_pi;
    d.tcerr = h->d_tcerr;
    d.U = h->U; d.V = h->V; d.W = h->W; d.P = h->P; d.GP = h->GP;
    d.US = h->US; d.VS = h->VS; d.WS = h->WS; d.PHI = h->PHI; d.PHIZ = h->PHIZ;
    const size_t se = spec_elems(h->cfg);
    if (h->mixed) {
        for (int f = 0; f < 6; ++f) {
            d.spec[f] = h->spec32[f];
            d.tmp[f] = h->fft.tmp32 + (size_t)f * se;
            d.phys[f] = h->phys32[f];
        }
        for (int f = 0; f < 3; ++f) d.src[f] = h->src32[f];
        d.tw_ny = h->fft.tw32_ny; d.tw_nx2 = h->fft.tw32_nx2; d.tw_nx = h->fft.tw32_nx;
    } else {
        double2* spec[6] = {h->U, h->V, h->W, h->US, h->VS, h->WS};
        for (int f = 0; f < 6; ++f) {
            d.spec[f] = spec[f];
            d.tmp[f] = h->fft.tmp + (size_t)f * se;
            d.phys[f] = h->phys[f];
        }
        d.src[0] = h->SU; d.src[1] = h->SV; d.src[2] = h->SW;
        d.fftfx = h->fft.fx ? 1 : 0;
        if (d.fftfx) {
            d.tw_ny = h->fft.twq_ny; d.tw_nx2 = h->fft.twq_nx2; d.tw_nx = h->fft.twq_nx;
        } else {
            d.tw_ny = h->fft.tw_ny; d.tw_nx2 = h->fft.tw_nx2; d.tw_nx = h->fft.tw_nx;
        }
    }
    d.ncol = h->sp.dealias ? std::min(h->sp.kx_max + 1, h->g.nxhp) : h->g.nxhp;
    if (d.ncol < 1) d.ncol = h->g.nxhp;
    ragged_geometry(d);
    return d;
}

int batch_fail(dns3d_batch* b, cudaError_t e, const char* what) {
    b->err = std::string(what) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? DNS3D_E_OOM : DNS3D_E_CUDA;
}

#define BK(b, call)                                               \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return batch_fail((b), e_, #call); \
    } while (0)

// Work maps of every stage for the group's current tile widths: runs ordered
// by descending nz (the costliest virtual blocks first), then uploaded with
// the descriptors.
int group_upload(dns3d_batch* b, dns3d_batch::Group& G) {
    const int n = (int)G.idx.size();
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return G.desc[a].g.nz > G.desc[c].g.nz; });
    std::vector<int> host((size_t)kRsStages * (2 * n + 1));
    for (int s = 0; s < kRsStages; ++s) {
        int* start = host.data() + (size_t)s * (2 * n + 1);
        int* ord = start + n + 1;
        start[0] = 0;
        size_t smem = 0;
        for (int j = 0; j < n; ++j) {
            const RunDesc& d = G.desc[order[j]];
            ord[j] = order[j];
            start[j + 1] = start[j] + ragged_blocks(s, G.mixed, d);
            smem = std::max(smem, ragged_smem(s, G.mixed, d));
        }
        G.total[s] = start[n];
        G.smem[s] = smem;
    }
    BK(b, cudaMemcpyAsync(G.d_desc, G.desc.data(), (size_t)n * sizeof(RunDesc), cudaMemcpyHostToDevice, b->stream));
    BK(b, cudaMemcpyAsync(G.d_map, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BK(b, cudaStreamSynchronize(b->stream));
    return DNS3D_OK;
}

cudaError_t group_launch(dns3d_batch::Group& G, int s, cudaStream_t st) {
    const int n = (int)G.idx.size();
    if (G.total[s] < 1) return cudaSuccess;
    StageMap map;
    map.start = G.d_map + (size_t)s * (2 * n + 1);
    map.order = map.start + n + 1;
    map.nruns = n;
    RunDesc* runs = G.d_desc;
    void* args[] = {&runs, &map};
    return cudaLaunchKernel((const void*)ragged_kernel(s, G.mixed, G.variant), dim3((unsigned)G.total[s]),
                            dim3(kStageThreads), args, G.smem[s], st);
}

// Stage tile widths for the group: each run's own widths, or one width for
// all runs, whichever launch is fastest (one warm launch, then three between
// events).  The stages timed write only work buffers, apart from the PI
// update in front of the vorticity tiles, whose controller states the caller
// restores.
int group_tune(dns3d_batch* b, dns3d_batch::Group& G) {
    const int n = (int)G.idx.size();
    cudaEvent_t e0, e1;
    BK(b, cudaEventCreate(&e0));
    BK(b, cudaEventCreate(&e1));
    int rc = DNS3D_OK;
    for (int s : {(int)kRsVort, (int)kRsVisc, (int)kRsPres}) {
        const int k = ragged_tile_kernel(s, G.mixed);
        const size_t lim = stage_smem_limit(ragged_kernel(s, G.mixed, G.variant));
        int best = -1;
        float best_ms = 0.f;
        for (int cand : {0, 4, 8, 16, 32}) {
            bool ok = true;
            for (int i = 0; i < n && ok; ++i) {
                const int w = cand ? cand : G.own_tc[(size_t)i * kTileKernels + k];
                G.desc[i].g.tc[k] = w;
                ok = ragged_smem(s, G.mixed, G.desc[i]) <= lim;
            }
            if (!ok) continue;
            if ((rc = group_upload(b, G))) break;
            cudaError_t ce = group_launch(G, s, b->stream);
            if (!ce) ce = cudaEventRecord(e0, b->stream);
            for (int r = 0; r < 3 && !ce; ++r) ce = group_launch(G, s, b->stream);
            if (!ce) ce = cudaEventRecord(e1, b->stream);
            if (!ce) ce = cudaEventSynchronize(e1);
            if (ce) {
                rc = batch_fail(b, ce, "batch tuning");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (best < 0 || ms < best_ms) {
                best = cand;
                best_ms = ms;
            }
        }
        if (rc) break;
        for (int i = 0; i < n; ++i)
            G.desc[i].g.tc[k] = best > 0 ? best : G.own_tc[(size_t)i * kTileKernels + k];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    return group_upload(b, G);
}

void batch_release(dns3d_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto& G : b->grp) {
        cudaFree(G.d_desc);
        cudaFree(G.d_map);
        for (auto ev : {G.lane_join, G.side_fork, G.side_join})
            if (ev) cudaEventDestroy(ev);
        for (auto st : {G.lane, G.side})
            if (st) cudaStreamDestroy(st);
    }
    for (auto ev : b->run_in) cudaEventDestroy(ev);
    for (auto ev : b->run_join) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
}

// One group's step on its lane: the nonlinear-term stages, then viscous and
// pressure tiles with (mixed form) the mode (0,0) chain forked beside them,
// then projection and walls.
cudaError_t group_capture(dns3d_batch::Group& G, int* launches) {
    cudaStream_t lane = G.lane, side = G.side;
    cudaError_t ce = cudaSuccess;
    auto stage = [&](int s, cudaStream_t st) {
        if (!ce && G.total[s] > 0) {
            ce = group_launch(G, s, st);
            *launches += 1;
        }
    };
    for (int s : {(int)kRsVort, (int)kRsFftYInv, (int)kRsFftC2R, (int)kRsProd, (int)kRsFftR2C, (int)kRsFftYFwd})
        stage(s, lane);
    if (G.mixed) {
        if (!ce) ce = cudaEventRecord(G.side_fork, lane);
        if (!ce) ce = cudaStreamWaitEvent(side, G.side_fork, 0);
        stage(kRsViscMean, side);
        stage(kRsPresMean, side);
        if (!ce) ce = cudaEventRecord(G.side_join, side);
    }
    stage(kRsVisc, lane);
    stage(kRsPresRhs, lane);
    stage(kRsPres, lane);
    if (G.mixed && !ce) ce = cudaStreamWaitEvent(lane, G.side_join, 0);
    stage(kRsCorr, lane);  // also writes the wall planes (RunDesc sp.bc_walls)
    return ce;
}

// One graph per step: fork -> (each group's stage launches on its lane, each
// loose run's step body on its own stream) -> join.
int batch_capture(dns3d_batch* b) {
    cudaGraph_t graph = nullptr;
    BK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = DNS3D_OK;
    int launches = 0;
    cudaError_t ce = cudaEventRecord(b->fork, b->stream);
    for (size_t gi = 0; gi < b->grp.size() && !ce; ++gi) {
        dns3d_batch::Group& G = b->grp[gi];
        ce = cudaStreamWaitEvent(G.lane, b->fork, 0);
        if (!ce) ce = group_capture(G, &launches);
        if (!ce) ce = cudaEventRecord(G.lane_join, G.lane);
        if (!ce) ce = cudaStreamWaitEvent(b->stream, G.lane_join, 0);
    }
    for (size_t j = 0; j < b->loose.size() && !ce && !rc; ++j) {
        const int i = b->loose[j];
        dns3d_handle* h = b->runs[i];
        ce = cudaStreamWaitEvent(h->stream, b->fork, 0);
        if (!ce) rc = run_step_body(h);
        launches += h->launches;
        if (!rc && !ce) ce = cudaEventRecord(b->run_join[i], h->stream);
        if (!rc && !ce) ce = cudaStreamWaitEvent(b->stream, b->run_join[i], 0);
    }
    cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
    if (rc || ce || ee) {
        if (graph) cudaGraphDestroy(graph);
        if (rc) {
            b->err = b->runs[b->loose.empty() ? 0 : b->loose[0]]->err;
            return rc;
        }
        return batch_fail(b, ce ? ce : ee, "batch capture");
    }
    cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ie) {
        b->graph = nullptr;
        return batch_fail(b, ie, "cudaGraphInstantiate (batch)");
    }
    BK(b, cudaGraphUpload(b->graph, b->stream));
    b->launches = launches;
    return DNS3D_OK;
}

int batch_create(dns3d_handle* const* runs, int nruns, int flags, dns3d_batch** out) {
    if (!runs || nruns < 1 || !out) return DNS3D_E_INVALID;
    *out = nullptr;
    for (int i = 0; i < nruns; ++i)
        if (!runs[i] || runs[i]->cfg.device != runs[0]->cfg.device) return DNS3D_E_INVALID;
    dns3d_batch* b = new dns3d_batch();
    b->runs.assign(runs, runs + nruns);
    b->device = runs[0]->cfg.device;
    int rc = DNS3D_OK;
    auto fail = [&](int code) {
        batch_release(b);
        delete b;
        return code;
    };
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(DNS3D_E_CUDA);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming))
        return fail(DNS3D_E_CUDA);
    b->run_in.assign(nruns, nullptr);
    b->run_join.assign(nruns, nullptr);
    for (int i = 0; i < nruns; ++i)
        if (cudaEventCreateWithFlags(&b->run_in[i], cudaEventDisableTiming) ||
            cudaEventCreateWithFlags(&b->run_join[i], cudaEventDisableTiming))
            return fail(DNS3D_E_CUDA);
    if (prepare_stage_kernels()) return fail(DNS3D_E_CUDA);
    // group the eligible runs by precision; a run whose stage launches would
    // not fit the stage kernels' shared memory keeps its own launches
    for (int i = 0; i < nruns; ++i) {
        dns3d_handle* h = runs[i];
        bool ok = ragged_eligible(h);
        RunDesc d{};
        if (ok) {
            d = make_desc(h);
            for (int s = 0; s < kRsStages && ok; ++s)
                ok = ragged_smem(s, h->mixed, d) <=
                     stage_smem_limit(ragged_kernel(s, h->mixed, h->mixed ? 0 : ragged_variant(d)));
        }
        if (!ok) {
            b->loose.push_back(i);
            continue;
        }
        const int variant = h->mixed ? 0 : ragged_variant(d);
        const int key = h->mixed ? 1 << 8 : variant;
        size_t gi = 0;
        while (gi < b->grp.size() && b->grp[gi].key != key) ++gi;
        if (gi == b->grp.size()) {
            b->grp.emplace_back();
            b->grp.back().key = key;
        }
        dns3d_batch::Group& G = b->grp[gi];
        G.mixed = h->mixed;
        G.variant = variant;
        G.idx.push_back(i);
        G.desc.push_back(d);
        for (int k = 0; k < kTileKernels; ++k) G.own_tc.push_back(d.g.tc[k]);
    }
    for (auto& G : b->grp) {
        const int n = (int)G.idx.size();
        if (cudaStreamCreateWithFlags(&G.lane, cudaStreamNonBlocking) ||
            cudaStreamCreateWithFlags(&G.side, cudaStreamNonBlocking) ||
            cudaEventCreateWithFlags(&G.lane_join, cudaEventDisableTiming) ||
            cudaEventCreateWithFlags(&G.side_fork, cudaEventDisableTiming) ||
            cudaEventCreateWithFlags(&G.side_join, cudaEventDisableTiming))
            return fail(DNS3D_E_CUDA);
        if (cudaMalloc(&G.d_desc, (size_t)n * sizeof(RunDesc)) ||
            cudaMalloc(&G.d_map, (size_t)kRsStages * (2 * n + 1) * sizeof(int)))
            return fail(DNS3D_E_OOM);
    }
    // the runs' queued work (state uploads, initial conditions) comes first
    for (int i = 0; i < nruns; ++i)
        if (cudaStreamSynchronize(runs[i]->stream)) return fail(DNS3D_E_CUDA);
    const char* env = std::getenv("DNS3D_AUTOTUNE");
    const bool tune = (flags & DNS3D_BATCH_TUNE) && !(env && std::strcmp(env, "0") == 0);
    std::vector<dns3d_pi_state> pis;
    if (tune) {
        pis.resize(nruns);
        for (int i = 0; i < nruns; ++i)
            if (cudaMemcpy(&pis[i], runs[i]->d_pi, sizeof(dns3d_pi_state), cudaMemcpyDeviceToHost))
                return fail(DNS3D_E_CUDA);
    }
    for (auto& G : b->grp) {
        if (G.idx.empty()) continue;
        rc = tune ? group_tune(b, G) : group_upload(b, G);
        if (rc) {
            for (dns3d_handle* h : b->runs) h->err = b->err;
            return fail(rc);
        }
    }
    if (tune) {
        for (int i = 0; i < nruns; ++i)
            if (cudaMemcpy(runs[i]->d_pi, &pis[i], sizeof(dns3d_pi_state), cudaMemcpyHostToDevice))
                return fail(DNS3D_E_CUDA);
        for (dns3d_handle* h : b->runs) h->phys_valid = 0;
    }
    if ((rc = batch_capture(b))) {
        for (dns3d_handle* h : b->runs) h->err = b->err;
        return fail(rc);
    }
    *out = b;
    return DNS3D_OK;
}

int batch_step(dns3d_batch* b, int nsteps) {
    BK(b, cudaSetDevice(b->device));
    for (size_t i = 0; i < b->runs.size(); ++i) {
        BK(b, cudaEventRecord(b->run_in[i], b->runs[i]->stream));
        BK(b, cudaStreamWaitEvent(b->stream, b->run_in[i], 0));
    }
    for (int s = 0; s < nsteps; ++s) {
        BK(b, cudaGraphLaunch(b->graph, b->stream));
        for (dns3d_handle* h : b->runs) {
            h->step += 1;
            h->time += h->cfg.dt;  // 3D:296
            h->phys_valid = 0;
        }
    }
    BK(b, cudaEventRecord(b->done, b->stream));
    for (dns3d_handle* h : b->runs) BK(b, cudaStreamWaitEvent(h->stream, b->done, 0));
    return DNS3D_OK;
}

}  // namespace

// ------------------------------------------------------------------ ensembles
struct dns3d_ensemble {
    std::vector<dns3d_handle*> runs;
    dns3d_batch* batch = nullptr;  // created at the first step
    int device = 0;
};

namespace {

void ensemble_release(dns3d_ensemble* e) {
    if (e->batch) {
        cudaStreamSynchronize(e->batch->stream);
        batch_release(e->batch);
        delete e->batch;
        e->batch = nullptr;
    }
    for (auto* h : e->runs) dns3d_destroy(h);
}

int ensemble_batch(dns3d_ensemble* e) {
    if (e->batch) return DNS3D_OK;
    return batch_create(e->runs.data(), (int)e->runs.size(), DNS3D_BATCH_TUNE, &e->batch);
}

}  // namespace

extern "C" {

int dns3d_batch_create(dns3d_handle* const* runs, int nruns, int flags, dns3d_batch** out) {
    return batch_create(runs, nruns, flags, out);
}

int dns3d_batch_step(dns3d_batch* b, int nsteps) {
    if (!b || nsteps < 0) return DNS3D_E_INVALID;
    return nsteps ? batch_step(b, nsteps) : DNS3D_OK;
}

int dns3d_batch_synchronize(dns3d_batch* b) {
    if (!b) return DNS3D_E_INVALID;
    BK(b, cudaSetDevice(b->device));
    BK(b, cudaStreamSynchronize(b->stream));
    return DNS3D_OK;
}

int dns3d_batch_query(dns3d_batch* b, int* done) {
    if (!b || !done) return DNS3D_E_INVALID;
    BK(b, cudaSetDevice(b->device));
    const cudaError_t e = cudaStreamQuery(b->stream);
    if (e == cudaErrorNotReady) {
        // not an error; make sure a later launch check cannot read it as one
        if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
        *done = 0;
        return DNS3D_OK;
    }
    BK(b, e);
    *done = 1;
    return DNS3D_OK;
}

int dns3d_batch_info(dns3d_batch* b, int* launches_per_step, int* ragged_runs) {
    if (!b) return DNS3D_E_INVALID;
    if (launches_per_step) *launches_per_step = b->launches;
    if (ragged_runs) {
        int n = 0;
        for (auto& G : b->grp) n += (int)G.idx.size();
        *ragged_runs = n;
    }
    return DNS3D_OK;
}

int dns3d_batch_destroy(dns3d_batch* b) {
    if (!b) return DNS3D_E_INVALID;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_release(b);
    delete b;
    return DNS3D_OK;
}

int dns3d_ensemble_create(const dns3d_config* cfgs, int nruns, dns3d_ensemble** out) {
    if (!cfgs || nruns < 1 || !out) return DNS3D_E_INVALID;
    *out = nullptr;
    for (int i = 0; i < nruns; ++i)
        if (cfgs[i].device != cfgs[0].device) return DNS3D_E_INVALID;
    dns3d_ensemble* e = new dns3d_ensemble();
    e->device = cfgs[0].device;
    for (int i = 0; i < nruns; ++i) {
        dns3d_handle* h = nullptr;
        const int rc = dns3d_create(&cfgs[i], &h);
        if (rc) {
            ensemble_release(e);
            delete e;
            return rc;
        }
        e->runs.push_back(h);
    }
    *out = e;
    return DNS3D_OK;
}

int dns3d_ensemble_destroy(dns3d_ensemble* e) {
    if (!e) return DNS3D_E_INVALID;
    cudaSetDevice(e->device);
    ensemble_release(e);
    delete e;
    return DNS3D_OK;
}

int dns3d_ensemble_size(dns3d_ensemble* e, int* nruns) {
    if (!e || !nruns) return DNS3D_E_INVALID;
    *nruns = (int)e->runs.size();
    return DNS3D_OK;
}

int dns3d_ensemble_run(dns3d_ensemble* e, int i, dns3d_handle** h) {
    if (!e || !h || i < 0 || i >= (int)e->runs.size()) return DNS3D_E_INVALID;
    *h = e->runs[i];
    return DNS3D_OK;
}

int dns3d_ensemble_step(dns3d_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return DNS3D_E_INVALID;
    dns3d_handle* h0 = e->runs[0];
    CK(h0, cudaSetDevice(e->device));
    if (nsteps == 0) return DNS3D_OK;
    int rc = ensemble_batch(e);
    if (!rc) rc = batch_step(e->batch, nsteps);
    if (rc) {
        if (e->batch) h0->err = e->batch->err;
        return rc;
    }
    CK(h0, cudaStreamSynchronize(e->batch->stream));
    return DNS3D_OK;
}

int dns3d_ensemble_step_timed(dns3d_ensemble* e, int nsteps, double* elapsed_ms) {
    if (!e || !elapsed_ms || nsteps < 1) return DNS3D_E_INVALID;
    dns3d_handle* h0 = e->runs[0];
    CK(h0, cudaSetDevice(e->device));
    int rc = ensemble_batch(e);
    if (rc) return rc;
    dns3d_batch* b = e->batch;
    // the runs' own queued work is ordered before the first event
    for (size_t i = 0; i < b->runs.size(); ++i) {
        CK(h0, cudaEventRecord(b->run_in[i], b->runs[i]->stream));
        CK(h0, cudaStreamWaitEvent(b->stream, b->run_in[i], 0));
    }
    cudaEvent_t a, c;
    CK(h0, cudaEventCreate(&a));
    CK(h0, cudaEventCreate(&c));
    CK(h0, cudaEventRecord(a, b->stream));
    rc = batch_step(b, nsteps);
    CK(h0, cudaEventRecord(c, b->stream));
    CK(h0, cudaEventSynchronize(c));
    float ms = 0.f;
    CK(h0, cudaEventElapsedTime(&ms, a, c));
    cudaEventDestroy(a);
    cudaEventDestroy(c);
    *elapsed_ms = ms;
    return rc;
}

int dns3d_ensemble_info(dns3d_ensemble* e, int* launches_per_step, int* ragged_runs) {
    if (!e) return DNS3D_E_INVALID;
    const int rc = ensemble_batch(e);
    if (rc) return rc;
    return dns3d_batch_info(e->batch, launches_per_step, ragged_runs);
}

const char* dns3d_strerror(int code) {
    switch (code) {
        case DNS3D_OK: return "ok";
        case DNS3D_E_INVALID: return "invalid argument or configuration";
        case DNS3D_E_OOM: return "device memory allocation failed";
        case DNS3D_E_SINGULAR: return "singular per-mode operator";
        case DNS3D_E_NONFINITE: return "non-finite value in the state";
        case DNS3D_E_CUDA: return "CUDA error";
        case DNS3D_E_UNSUPPORTED: return "unsupported grid size or option";
        case DNS3D_E_IO: return "input file could not be read or parsed";
        case DNS3D_E_NODEVICE: return "no CUDA device";
        case DNS3D_E_TIMEOUT: return "timed out";
        case DNS3D_E_CANCELLED: return "request cancelled";
        default: return "unknown error";
    }
}

const char* dns3d_last_error(dns3d_handle* h) {
    if (!h) return "";
    return h->err.c_str();
}

}  // extern "C"

// Internal declarations shared by the translation units of libdns3d_gpu.so.
//
// Data layout in HBM (all FP64):
//   spectral field : double2 [nz][ny][nxhp]   (nxhp = nx/2+1, FFTW r2c order,
//                    kx fastest; the same memory order as the reference's
//                    complex(nxhp,ny) planes, DNS_pressure_BC_3D.f90:1442)
//   physical field : double  [nz][ny][nx]     (Fortran u(nx,ny,nz))
//   z-operators    : double  [nz][nz] row-major, A[z][z'] (applied as A . f(:))
//   per-mode inverses : double [nq][nz][nz] stored TRANSPOSED, Ainv^T[q][z'][z],
//                    so that threads indexed by the output row z read
//                    consecutive addresses for a fixed z'.
// A "mode" m = ky*nxhp + kx indexes one complex column of length nz; a plane
// holds nm = nxhp*ny modes.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dns3d_capi.h"

namespace dns3d {

constexpr int kMaxFields = 8;
constexpr int kMaxStages = 12;

template <typename C>
struct FieldsT {
    C* p[kMaxFields];
};
using Fields = FieldsT<double2>;    // FP64 spectral
using RFields = FieldsT<double>;    // FP64 physical
using FFields = FieldsT<float2>;    // FP32 spectral
using FRFields = FieldsT<float>;    // FP32 physical

// Radix schedule of one complex FFT length (Stockham autosort, radices 4/2/3).
struct FftPlan1D {
    int n;
    int nstages;
    int radix[kMaxStages];
};

FftPlan1D make_plan(int n);
bool fft_length_supported(int n);

template <typename T> struct Cx;
template <> struct Cx<double> { using type = double2; };
template <> struct Cx<float> { using type = float2; };

// Grid constants passed by value to kernels.
// Mode-tile kernels whose tile width (mode columns per CTA) is tunable; the
// results do not depend on it (every output is one thread's fixed-order sum).
enum TileKernel { kTileVort = 0, kTileVisc, kTilePres, kTileCorr, kTileDiv, kTileVortM, kTileViscM, kTilePresM,
                  kTileKernels };

struct GridDev {
    int nx, ny, nz, nxh, nxhp, nm;
    int nkyu;            // ny/2 + 1 unique |ky|
    double inv_nxny;     // 1/(nx*ny), c2r normalisation
    int tc[kTileKernels];  // chosen tile widths (0: built-in heuristic)
    int refine;            // mixed pressure: keeps its FP64 right-hand side for the refinement step
};

// Maps a spectral mode (ky, kx) to the index of its per-mode operator: the
// operators depend on kx^2 + ky^2 only, so ky and ny-ky share one.
__host__ __device__ inline int mode_q(int ky, int kx, int ny, int nxhp) {
    int kya = ky <= ny / 2 ? ky : ny - ky;
    return kya * nxhp + kx;
}

// ---------------------------------------------------------------- fft.cu
// Batched real 2D transforms over planes of the listed fields.  c2r keeps
// FFTW's semantics for non-Hermitian input: inverse c2c along y, then a 1D
// c2r along x that ignores Im of the kx=0 and kx=nx/2 entries; output scaled
// by 1/(nx*ny) (fftw3_dns_module.f90:127-130).
struct FftCtx {
    FftPlan1D py;        // length ny complex
    FftPlan1D px2;       // length nx/2 complex (packed real transform)
    double2* tw_ny;      // e^{-2 pi i t/ny}, t < ny
    double2* tw_nx2;     // e^{-2 pi i t/(nx/2)}
    double2* tw_nx;      // e^{-2 pi i t/nx}, t < nx/2+1
    float2* tw32_ny;     // FP32 copies of the tables (mixed path)
    float2* tw32_nx2;
    float2* tw32_nx;
    longlong2* twq_ny = nullptr;   // Q62 integer copies (fixed-point FP64 transforms)
    longlong2* twq_nx2 = nullptr;
    longlong2* twq_nx = nullptr;
    // FP64 transforms in 64-bit fixed point on the integer pipes (fft_ct.cu);
    // set for grids with compile-time kernels unless DNS3D_FFT_FP64=1 keeps
    // them on the FP64 pipe
    bool fx = false;
    double2* tmp;        // spectral scratch for nf fields
    float2* tmp32 = nullptr;  // FP32 spectral scratch (mixed path)
    int tmp_fields;
    bool use_ct = false;  // the grid's lengths have compile-time kernels (fft_ct.cu)
    // optional per-launch hook (profiling): called after each kernel launch
    void (*hook)(void*, const char*) = nullptr;
    void* hook_ctx = nullptr;
};
// Compile-time-length plane transforms (fft_ct.cu) for ny in {16..512} and
// nx/2 in {16..256} of the form 2^a 3^b; fft_ct_supported tells which grids.
bool fft_ct_supported(int ny, int nxh);
template <int SIGN, typename C>
cudaError_t fft_ct_y(FieldsT<C> src, FieldsT<C> dst, const GridDev& g, int nplanes, int ncol, int nf, const C* tw,
                     cudaStream_t s);
template <typename T>
cudaError_t fft_ct_c2r_x(FieldsT<typename Cx<T>::type> src, FieldsT<T> dst, const GridDev& g, int nrows, int nf,
                         const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s);
template <typename T>
cudaError_t fft_ct_r2c_x(FieldsT<T> src, FieldsT<typename Cx<T>::type> dst, const GridDev& g, int nrows, int nf,
                         const typename Cx<T>::type* tw_n, const typename Cx<T>::type* tw_nx, cudaStream_t s);

// The FP64 passes of fft_ct in block fixed point (Q62 twiddle tables).
template <int SIGN>
cudaError_t fft_fx_y(Fields src, Fields dst, const GridDev& g, int nplanes, int ncol, int nf, const longlong2* tw,
                     cudaStream_t s);
// dst2 (entries may be null): a second destination of the same values
cudaError_t fft_fx_c2r_x(Fields src, RFields dst, RFields dst2, const GridDev& g, int nrows, int nf,
                         const longlong2* tw_n, const longlong2* tw_nx, cudaStream_t s);
// host_src: src is host memory mapped for the device (plain loads instead of
// bulk copies)
cudaError_t fft_fx_r2c_x(RFields src, Fields dst, const GridDev& g, int nrows, int nf, const longlong2* tw_n,
                         const longlong2* tw_nx, bool host_src, cudaStream_t s);

cudaError_t fft_setup(FftCtx& ctx, const GridDev& g);
void fft_release(FftCtx& ctx);
// spec[f] (spectral, read only) -> phys[f]; uses the ctx.tmp slots slot0 ..
// slot0 + nf - 1 (at most tmp_fields), so that two calls on different slots can
// run concurrently.
cudaError_t fft_c2r(const FftCtx& ctx, const GridDev& g, Fields spec, RFields phys, int nf,
                    int nplanes, cudaStream_t s, int slot0 = 0);
// The same into phys[f] and into copy[f] as well (host memory the device
// can address, for example), in one pass; only where ctx.fx is set
// (cudaErrorNotSupported otherwise).
cudaError_t fft_c2r_copy(const FftCtx& ctx, const GridDev& g, Fields spec, RFields phys, RFields copy, int nf,
                         int nplanes, cudaStream_t s);
// phys[f] -> spec[f].  With ncol > 0 only the kx < ncol columns of spec are
// completed (the others keep the x transform's output): for sources that the
// 2/3 filter truncates at kx_max = ncol - 1 anyway.
cudaError_t fft_r2c(const FftCtx& ctx, const GridDev& g, RFields phys, Fields spec, int nf,
                    int nplanes, cudaStream_t s, int ncol = 0, bool host_src = false);
// FP32 versions (same transform definitions), scratch ctx.tmp32.
cudaError_t fft_c2r32(const FftCtx& ctx, const GridDev& g, FFields spec, FRFields phys, int nf,
                      int nplanes, cudaStream_t s);
cudaError_t fft_r2c32(const FftCtx& ctx, const GridDev& g, FRFields phys, FFields spec, int nf,
                      int nplanes, cudaStream_t s, int ncol = 0);

// ---------------------------------------------------------------- step.cu
struct StepParams {
    double dt;
    double inv_dt;        // 1/dt, formed once on the host (an FP64 division is a long sequence on this GPU)
    double cn_fac;        // 0.5*dt/Re if Crank-Nicolson else 0 (3D:1374)
    double helm_f;        // theta*dt/Re (3D:1459)
    double forcing_scale; // nx*ny: physical constant -> (0,0) coefficient
    int dealias;          // use_dealias_23_rule
    int kx_max, ky_max;   // 2/3 limits (3D:1169-1170)
    int weak_form;        // use_weak_form_divergence
    int rhs_only;         // viscous/pressure kernels: write the right-hand sides (for jacgs), not the solutions
    int cn_identity;      // Crank-Nicolson: explicit half folded into the implicit solve (step.cu)
    int bc_walls;         // projection: write the wall planes of u, v, w as zero (apply_boundary_conditions_3d
                          // fused into it; set by the fused step, not by the five-stage calls)
    int refine;           // mixed pressure: one step of iterative refinement (dns3d_config::poisson_refinement)
};

// z-operators in parity-folded form (see step.cu): for nz levels,
// he = nz - nz/2 even-part and ho = nz/2 odd-part values per column.
//   antisymmetric D: De [he][ho] (acts on the odd part), Do [ho][he]
//   symmetric A:     Ae [he][he], Ao [ho][ho]
// Per-mode inverses: per q, [GeT (he*he) | GoT (ho*ho)], each block stored
// transposed.
struct Ops {
    int he, ho;
    double* D1e; double* D1o;   // (2/ybar) d1
    double* D2e; double* D2o;   // (2/ybar)^2 d2
    double* W1e; double* W1o;   // zwts[m]*(2/ybar)*d1(m,z) as [z][m] (weak-form vertical part)
    double* wh;      // zwts * ybar/2           [nz]
    double* zw;      // zwts                    [nz]
    double* S0;      // helm_f * S[z][0]        [nz]
    double* Sn;      // helm_f * S[z][nz-1]     [nz]
    double* xw;      // [nxhp]
    double* yw;      // [ny]
    double* ksq;     // xsq+ysq per unique q     [nq]
    double* S;       // stiffness (2/ybar) sum_m d1(m,k) d1(m,n) zwts(m), [nz][nz] (jacgs)
    double* HinvF;   // folded Helmholtz inverses      [nq][he*he + ho*ho]
    double* PinvF;   // folded Poisson inverses        [nq][he*he + ho*ho]
    double* PpinT;   // pinned (0,0) Poisson inverse, unfolded, transposed [nz][nz]
    // PinvF in 58-bit fixed point for the solve on the integer pipes (FP64
    // runs with the tensor-core forms), or null: entry (j, k) of a folded
    // block round(G[k][j] 2^(58 - e_k)) in PinvF's layout but with a per-q
    // stride of fx_qstride (even), row exponents e_k [nq][he + ho] (block
    // E's rows, then block O's)
    const long long* PinvI;
    const int* PinvE;
    int nq;
    // tensor-core form of HinvF (tc.cuh), or null: FP16 digit slices
    // [nq][tc_q_halves] of 2 G[i][j] w_j and row exponents [nq][m8] (rows i
    // of both blocks share one); tcTau [2][he]: the lifting coefficients of
    // the weight-free folded right-hand sides, (S0_k + Sn_k) / (2 w_k) and
    // (S0_k - Sn_k) / (2 w_k) (the unpaired mid level: S0 / (2 w))
    const __half* tcA;
    const int* tcE;
    const double* tcTau;
    // tensor-core digit image of the folded D1 ([[0, De], [Do, 0]]), or null
    const __half* tcD;
    const int* tcDE;
    // failure-detection test: the tensor-core kernels withhold their MMA
    // commit and poll their completion barrier only 2^10 times, so the bounded
    // wait runs out and reports its status (0 in normal runs)
    int tc_stall;
};

// Mixed-precision operators (FP32): folded D for the nonlinear term and the
// eigenbasis of the interior Helmholtz problem S_II V = M_II V Lambda
// (ni = nz - 2 interior levels).
// Mixed-precision operators (FP32): folded D for the nonlinear term, the
// eigenbasis of the interior Helmholtz problem S_II V = M_II V Lambda
// (ni = nz - 2 interior levels) and of the full Neumann problem
// S V' = M V' Lambda'.  The GEMM operands are stored with their output-row
// index innermost and padded to a multiple of 4 (nip, nzp) with zeros, so one
// float4 load feeds four output rows.
struct MixedOps {
    float* D1e; float* D1o;  // folded (2/ybar) d1, FP32
    // folded (2/ybar) d1 and weak-form operator as double-float pairs
    // (hi = (float)x, lo = (float)(x - hi)) for the divergence right-hand side
    float2* D1e_df; float2* D1o_df;
    float2* W1e_df; float2* W1o_df;
    int nzp;                 // nz rounded up to a multiple of 4
    // interior eigenbasis, folded: the interior problem is centro-symmetric, so
    // its eigenvectors are even or odd and the basis splits into an even block
    // (hei = ni - ni/2 rows) and an odd block (hoi = ni/2), padded to pe4, po4.
    // Forward: ut_even = Ae [s; u_mid], ut_odd = Ao d (s, d = pair sums and
    // differences of the interior values); back: pe = Be y_even, po = Bo y_odd,
    // x_i = pe_i + po_i, x_{ni-1-i} = pe_i - po_i, x_mid = pe_mid.
    int hei, hoi, pe4, po4;
    float* AeT;              // [hei][pe4]  Ae[j][i] stored at [i][j]
    float* AoT;              // [hoi][po4]
    float* BeT;              // [hei][pe4]  Be[i][j] stored at [j][i]
    float* BoT;              // [hoi][po4]
    float* lam;              // [pe4 + po4] eigenvalues (even block, then odd block)
    float* s0;               // [pe4 + po4] V^T S_I1 in the same order
    float* sn;               // [pe4 + po4] V^T S_In
    // Neumann eigenbasis S V' = M V' Lambda', folded like the interior one:
    // even eigenvectors (he of them) act on the folded sums of the right-hand
    // side, odd ones (ho) on the differences; D V' maps even eigenvectors to
    // odd functions and odd ones to even functions.  Row blocks padded to
    // phe4 = pad4(he), pho4 = pad4(ho); every matrix is stored with its
    // output index innermost:
    //   PAe [he][phe4]: phi~e_j = sum_i PAe[i][j] s_i   (forward, even)
    //   PAo [ho][pho4]: phi~o_j = sum_i PAo[i][j] d_i   (forward, odd)
    //   PBe [he][phe4]: pe_i = sum_j PBe[j][i] phi~e_j  (back, even part)
    //   PBo [ho][pho4]: po_i = sum_j PBo[j][i] phi~o_j  (back, odd part)
    //   PDe [ho][phe4]: (dphi/dz) even part from phi~o; PDo [he][pho4]: odd part from phi~e
    int phe4, pho4;
    float* PAe; float* PAo; float* PBe; float* PBo; float* PDe; float* PDo;
    // PAe, PAo with input row i scaled by 2 w_i / dt: the forward solve of the
    // strong-form right-hand side, which is then formed without the weights
    // and the 1/dt (pressure_mixed_body)
    float* PAeS; float* PAoS;
    float* plame;            // [phe4] eigenvalues of the even block
    float* plamo;            // [pho4] eigenvalues of the odd block
    // folded stiffness S (symmetric fold of ops.S) as double-float pairs, for
    // the FP64-accurate residual of the refinement: Se [he][he], So [ho][ho]
    float2* Se_df; float2* So_df;
};

struct PIParams {
    int method;
    int istart;
    int update_freq;
    double target_dpdx, target_ub, gain, re, dt;
    double inv_nxny_wsum;   // 1/(nx*ny*sum(zwts))
};

// Sets the dynamic shared-memory limits of the kernels below (call once per
// grid, outside stream capture).
cudaError_t prepare_step_kernels(const GridDev& g);
// Tile width of a mode-tile kernel: g.tc[k] if set, else the heuristic; and
// whether width tc fits the kernel's shared-memory limit.
int tile_width(const GridDev& g, int k);
bool tile_fits(const GridDev& g, int k, int tc);
cudaError_t launch_pi_update(const GridDev& g, const Ops& ops, const PIParams& pp,
                             const double2* U, dns3d_pi_state* pi, cudaStream_t s);
cudaError_t launch_vorticity(const GridDev& g, const Ops& ops, const double2* U,
                             const double2* V, const double2* W, double2* OX, double2* OY,
                             double2* OZ, cudaStream_t s);
cudaError_t launch_products(const GridDev& g, RFields in6, RFields out3, cudaStream_t s);
cudaError_t launch_viscous(const GridDev& g, const Ops& ops, const StepParams& sp,
                           Fields F, Fields Src, const double2* GP,
                           const dns3d_pi_state* pi, Fields Out, cudaStream_t s);
// The Crank-Nicolson viscous step with the folded inverses applied on the
// tensor cores in emulated FP64 (ops.tcA set, sp.cn_identity); err receives 1
// if a tensor-core completion wait ran out.
cudaError_t launch_viscous_tc(const GridDev& g, const Ops& ops, const StepParams& sp, Fields F, Fields Src,
                              const double2* GP, const dns3d_pi_state* pi, Fields Out, int* err, cudaStream_t s);
size_t viscous_tc_smem(const GridDev& g);
bool viscous_tc_fits(const GridDev& g);
// The vorticity with the z-derivatives D1.u, D1.v on the tensor cores in
// emulated FP64 (ops.tcD set); err as for launch_viscous_tc.
cudaError_t launch_vorticity_tc(const GridDev& g, const Ops& ops, const double2* U, const double2* V,
                                const double2* W, double2* OX, double2* OY, double2* OZ, int* err, cudaStream_t s);
// solve_pressure_3d (strong form) with D1.w* on the tensor cores (ops.tcD
// set): the right-hand side into PHI, then the per-mode Poisson solve in place
cudaError_t launch_pressure_tc(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                               const double2* VS, const double2* WS, double2* PHI, int* err, cudaStream_t s);
// pressure_correction_3d with D1.phi on the tensor cores (ops.tcD set)
cudaError_t launch_correction_tc(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                 const double2* VS, const double2* WS, const double2* PHI, double2* U, double2* V,
                                 double2* W, double2* P, double2* GP, int* err, cudaStream_t s);
size_t vorticity_tc_smem(const GridDev& g);
bool vorticity_tc_fits(const GridDev& g);
cudaError_t launch_vorticity_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops,
                                   const double2* U, const double2* V, const double2* W, FFields out,
                                   cudaStream_t s);
cudaError_t launch_pressure_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops,
                                  const StepParams& sp, const double2* US, const double2* VS,
                                  const double2* WS, double2* PHI, double2* PHIZ, cudaStream_t s);
cudaError_t launch_correction_mixed(const GridDev& g, const Ops& ops, const StepParams& sp,
                                    const double2* US, const double2* VS, const double2* WS,
                                    const double2* PHI, const double2* PHIZ, double2* U, double2* V,
                                    double2* W, double2* P, double2* GP, cudaStream_t s);
cudaError_t launch_products32(const GridDev& g, FRFields in6, FRFields out3, cudaStream_t s);
cudaError_t launch_viscous_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops,
                                 const StepParams& sp, Fields F, FFields Src, const double2* GP,
                                 Fields Out, cudaStream_t s);
// jacgs (Jacobi-preconditioned CG) on the right-hand sides the viscous and
// pressure kernels left in place with StepParams::rhs_only: every non-pinned
// Poisson system (S + k^2 w ybar/2) phi = -b and every interior Helmholtz
// system, one warp per real system, at most 500 iterations, stopping at
// residual <= tol * initial residual.
cudaError_t launch_pcg_poisson(const GridDev& g, const Ops& ops, double2* PHI, double tol, cudaStream_t s);
cudaError_t launch_pcg_helmholtz(const GridDev& g, const Ops& ops, const StepParams& sp, Fields Out, double tol,
                                 cudaStream_t s);
// jst4 stage state: out = F + coef * mask(S) with the wall levels zeroed.
template <typename SrcC>
cudaError_t launch_rk_stage(const GridDev& g, const StepParams& sp, double coef, Fields F, FieldsT<SrcC> Src,
                            Fields Out, cudaStream_t s);
// The mixed form's mode (0,0) in FP64 (independent of the mode tiles above).
cudaError_t launch_viscous_mean_mode(const GridDev& g, const Ops& ops, const StepParams& sp, Fields F,
                                     FFields Src, const double2* GP, const dns3d_pi_state* pi,
                                     Fields Out, cudaStream_t s);
cudaError_t launch_pressure_mean_mode(const GridDev& g, const Ops& ops, const StepParams& sp,
                                      const double2* US, const double2* VS, const double2* WS,
                                      double2* PHI, double2* PHIZ, cudaStream_t s);
cudaError_t launch_pressure(const GridDev& g, const Ops& ops, const StepParams& sp,
                            const double2* US, const double2* VS, const double2* WS,
                            double2* PHI, cudaStream_t s);
cudaError_t launch_correction(const GridDev& g, const Ops& ops, const StepParams& sp,
                              const double2* US, const double2* VS, const double2* WS,
                              const double2* PHI, double2* U, double2* V, double2* W,
                              double2* P, double2* GP, cudaStream_t s);
cudaError_t launch_apply_bc(const GridDev& g, double2* U, double2* V, double2* W,
                            cudaStream_t s);
cudaError_t launch_divergence(const GridDev& g, const Ops& ops, const double2* U,
                              const double2* V, const double2* W, double2* DIV,
                              cudaStream_t s);
cudaError_t launch_grad_walls(const GridDev& g, const Ops& ops, const double2* P,
                              double2* GP, cudaStream_t s);
// Reductions over physical fields.  out[0..3] = max|u|, max|v|, max|w|,
// sum 0.5(u^2+v^2+w^2) zwts[k]; partial buffer must hold 4*nblocks doubles.
cudaError_t launch_diag_reduce(const GridDev& g, const Ops& ops, const double* u,
                               const double* v, const double* w, double* partial,
                               int nblocks, double* out, cudaStream_t s);
// controller state (8 doubles) and the (0,0) modes of u, v, w (3 nz complex)
// into out, for one copy back
cudaError_t launch_diag_gather(const GridDev& g, const double2* U, const double2* V, const double2* W,
                               const dns3d_pi_state* pi, double* out, cudaStream_t s);
cudaError_t launch_maxabs(const GridDev& g, const double* f, size_t n, double* partial,
                          int nblocks, double* out, cudaStream_t s);
cudaError_t launch_nonfinite_check(const double2* f, size_t n, int* flag, cudaStream_t s);

// ---------------------------------------------------------------- setup.cu
// Build the per-mode operator inverses on the device by Gauss-Jordan with
// partial pivoting.  info[0] receives 1 + index of the first singular matrix.
// Outputs: HinvF/PinvF folded per q (layout of Ops), PpinT the unfolded
// transposed inverse of the pinned (0,0) Poisson operator.
cudaError_t build_inverses(const GridDev& g, const double* S, const double* wh,
                           double helm_f, const double* ksq, int nq, double* HinvF,
                           double* PinvF, double* PpinT, int* info, cudaStream_t s);
// The 58-bit fixed-point image of the folded Poisson inverses (Ops::PinvI, PinvE).
cudaError_t build_fixed_rows(const GridDev& g, const double* PinvF, int nq, long long* PinvI, int* PinvE,
                             cudaStream_t s);

// Residual of the Galerkin Poisson system of the last pressure step: max |b(u*)
// - P phi| and max |b| (bits of non-negative doubles, out[0], out[1]).
cudaError_t launch_poisson_residual(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                    const double2* VS, const double2* WS, const double2* PHI,
                                    unsigned long long* out, cudaStream_t s);

// Digit slices (FP16) and row exponents of the folded per-mode inverses invF
// ([nq][he*he + ho*ho], the layout of Ops::HinvF) with their columns scaled
// by 2 wfold[j] (the folded weights, device [he]) for the tensor-core solve
// (tc.cuh); slices [nq][tc_q_halves], rowexp [nq][m8], rows i of both blocks
// sharing one exponent.
cudaError_t build_tc_slices(const GridDev& g, const double* invF, const double* wfold, int nq, __half* slices,
                            int* rowexp, cudaStream_t s);

// Digit image ([kTcSlices][block E, block O] FP16, tc_blocks(t, true); rowexp
// [m8]) of the folded z-derivative [[0, De], [Do, 0]] for the tensor-core
// contractions (tc.cuh).
cudaError_t build_tc_anti_image(const GridDev& g, const double* De, const double* Do, __half* image, int* rowexp,
                                cudaStream_t s);

// The integer-pipe conversions (cvt.cuh) against the hardware ones on n
// pseudo-random values; mismatches counted.
cudaError_t check_conversions(long long n, unsigned long long* mismatches);

// Dense FP64 FMA throughput probe (TFLOP/s).
cudaError_t measure_fp64_tflops(int device, double* tflops);

// ---------------------------------------------------------------- lgl.cpp
void lgl_nodes_weights(int n, std::vector<double>& x, std::vector<double>& w);
void lgl_diff_matrix(const std::vector<double>& x, bool guard, std::vector<double>& d);
// Symmetric eigen-decomposition (cyclic Jacobi, FP64): a (n x n, row-major,
// destroyed) = Y diag(w) Y^T; Y returned row-major with eigenvectors as columns,
// eigenvalues ascending.
void jacobi_eigen(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& y);

// ---------------------------------------------------------------- namelist.cpp
int read_namelist_file(const char* path, dns3d_config* cfg);

}  // namespace dns3d

// Spectral-resident kernels of the time step (FP64).
//
// The reference works in physical space and round-trips every derivative
// through r2c/c2r per plane (compute_derivatives_3d, DNS_pressure_BC_3D.f90:
// 2321-2407).  For a real field f with spectrum F those round trips are the
// exact spectral maps
//   DX(F) = i xw(kx) F,  except the kx = nx/2 column, which the c2r discards
//   DY(F) = i yw(ky) F,  except (ky = ny/2, kx in {0, nx/2}), likewise
//   Dz(F) = (2/ybar) d1 . F(:)   (the physical d1 column product commutes with
//                                  the x-y transforms)
// so the state (u, v, w, p_total) is kept as spectra and only the nonlinear
// product is formed in physical space.
//
// "Mode-tile" kernels: one CTA owns TC consecutive modes m = ky*nxhp + kx and
// all nz levels of them, so z-contractions (nz x nz operator times a column)
// and the per-mode solves run out of shared memory with coalesced HBM access
// along m.
#include "dns3d_internal.cuh"
#include "ragged.cuh"
#include "tc.cuh"
#include "cvt.cuh"

#include <algorithm>
#include <climits>

namespace dns3d {
namespace {

__device__ __forceinline__ double2 i_times(double a, double2 f) {  // (i a) * f
    return make_double2(-a * f.y, a * f.x);
}

struct ModeInfo {
    int ky, kx;
    double ax, ay;  // DX / DY multipliers with the Nyquist rules applied
};

__device__ __forceinline__ ModeInfo mode_info(const GridDev& g, int m, const double* __restrict__ xw,
                                              const double* __restrict__ yw) {
    ModeInfo mi;
    mi.ky = m / g.nxhp;
    mi.kx = m - mi.ky * g.nxhp;
    mi.ax = (mi.kx == g.nxh) ? 0.0 : __ldg(&xw[mi.kx]);
    mi.ay = (mi.ky == g.ny / 2 && (mi.kx == 0 || mi.kx == g.nxh)) ? 0.0 : __ldg(&yw[mi.ky]);
    return mi;
}

// Field pointer `i` of a by-value FieldsT, selected without a dynamic index
// into the parameter block (which would copy the array to local memory).
template <typename P> __device__ __forceinline__ P* fptr(const FieldsT<P>& f, int i) {
    P* r = f.p[0];
#pragma unroll
    for (int k = 1; k < kMaxFields; ++k)
        if (i == k) r = f.p[k];
    return r;
}

// ------------------------------------------------------------------ PI / forcing
// update_pressure_gradient_3d (3D:2488-2549) called with the namelist istart
// (3D:1118), and calculate_bulk_velocity_3d (3D:2434-2464) from the (0,0) mode:
// sum_ij u(i,j,k) = Re U[k][0][0].
// The CTA's threads load the nz values of the mean mode in parallel (one
// 16-byte load per level, a plane apart); thread 0 then sums them in level
// order and runs the controller.  Every thread of the CTA must call it.
__device__ __forceinline__ void pi_update_body(GridDev g, const double* __restrict__ zw, PIParams pp,
                                               const double2* __restrict__ U, dns3d_pi_state* pi, int bx) {
    if (bx != 0) return;
    if (pp.method == 1) {
        if (threadIdx.x == 0) pi->current_pressure_gradient = pp.target_dpdx;
        return;
    }
    if (pp.method != 2) return;
    if (pp.istart % pp.update_freq != 0) return;
    __shared__ double col[129];  // Re U at mode (0,0), every level (nz <= 129)
    for (int k = threadIdx.x; k < g.nz; k += blockDim.x) col[k] = U[(size_t)k * g.nm].x;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double vol = 0.0;
    for (int k = 0; k < g.nz; ++k) vol = fma(col[k], zw[k], vol);
    const double ub = vol * pp.inv_nxny_wsum;
    pi->current_bulk_velocity = ub;
    const double err = pp.target_ub - ub;
    pi->bulk_velocity_error = err;
    const double kp = pp.gain, ki = 0.05 * pp.gain;
    const double unclamped = 3.0 / pp.re + kp * err + ki * pi->bulk_velocity_error_integral;
    const double clamped = fmax(0.0, fmin(10.0, unclamped));
    if (fabs(clamped - unclamped) < 1.0e-12) {
        if (pp.istart <= pp.update_freq)
            pi->bulk_velocity_error_integral += err * pp.dt;
        else
            pi->bulk_velocity_error_integral += 0.5 * pp.dt * (pi->bulk_velocity_error_prev + err);
    }
    pi->bulk_velocity_error_prev = err;
    pi->current_pressure_gradient = clamped;
    pi->pressure_gradient_sum += clamped;
    pi->pressure_gradient_count += 1;
    pi->avg_pressure_gradient = pi->pressure_gradient_sum / (double)pi->pressure_gradient_count;
}

__global__ void k_pi_update(GridDev g, const double* __restrict__ zw, PIParams pp,
                            const double2* __restrict__ U, dns3d_pi_state* pi) {
    pi_update_body(g, zw, pp, U, pi, blockIdx.x);
}

// ------------------------------------------------------------------ parity folding
// The LGL operators are centro-symmetric (D2, the Helmholtz and Poisson
// inverses: A[n-1-i][n-1-j] = A[i][j]) or centro-antisymmetric (D, the
// weak-form operator).  With s_i = x_i + x_{n-1-i}, d_i = x_i - x_{n-1-i}
// (i < n/2) and the middle value x_m when nz is odd, a column splits into an
// even part fe = [s; x_m] (he = nz - nz/2 values) and an odd part fo = d
// (ho = nz/2 values), and every operator becomes two half-size blocks:
//   symmetric A:  ye = Ae fe,  yo = Ao fo
//   antisym.  D:  ye = De fo,  yo = Do fe
//   y_i = ye_i + yo_i,  y_{n-1-i} = ye_i - yo_i,  y_m = ye_m
// which halves the FP64 multiply-adds of every z-contraction.  The blocks are
// built from the full operators (host: dns3d_create; device: the inverses).

// tile = [fe (he x tc) | fo (ho x tc)] of field src, modes m0 .. m0+tc-1.
__device__ __forceinline__ void fold_load(double2* tile, const double2* __restrict__ src, const GridDev& g,
                                          int m0, int tc, int he, int ho) {
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        double2 fe = make_double2(0.0, 0.0), fo = fe;
        if (m < g.nm) {
            const double2 a = src[(size_t)k * g.nm + m];
            if (k < ho) {
                const double2 b = src[(size_t)(g.nz - 1 - k) * g.nm + m];
                fe = make_double2(a.x + b.x, a.y + b.y);
                fo = make_double2(a.x - b.x, a.y - b.y);
            } else {
                fe = a;
            }
        }
        tile[t] = fe;
        if (k < ho) tile[(he + k) * tc + c] = fo;
    }
}

// ye = sum_j E[k][j] * in[j] over j < len (E row-major with leading dim len);
// in is a folded tile part with column stride tc.
__device__ __forceinline__ double2 fold_dot(const double* __restrict__ erow, const double2* in, int len, int tc,
                                            int c) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
    for (int j = 0; j < len; ++j) {
        const double e = __ldg(&erow[j]);
        const double2 a = in[j * tc + c];
        acc.x = fma(e, a.x, acc.x);
        acc.y = fma(e, a.y, acc.y);
    }
    return acc;
}

// Antisymmetric operator (De [he][ho], Do [ho][he]) on a folded tile: returns
// the output pair (y at z = k, y at z = nz-1-k); for the middle row only .a.
struct Pair {
    double2 a, b;
};
__device__ __forceinline__ Pair anti_apply(const double* __restrict__ De, const double* __restrict__ Do,
                                           const double2* tile, int k, int c, int tc, int he, int ho) {
    const double2 ye = fold_dot(De + (size_t)k * ho, tile + he * tc, ho, tc, c);
    Pair p;
    if (k < ho) {
        const double2 yo = fold_dot(Do + (size_t)k * he, tile, he, tc, c);
        p.a = make_double2(ye.x + yo.x, ye.y + yo.y);
        p.b = make_double2(ye.x - yo.x, ye.y - yo.y);
    } else {
        p.a = ye;
        p.b = ye;
    }
    return p;
}
__device__ __forceinline__ Pair sym_apply(const double* __restrict__ Ae, const double* __restrict__ Ao,
                                          const double2* tile, int k, int c, int tc, int he, int ho) {
    const double2 ye = fold_dot(Ae + (size_t)k * he, tile, he, tc, c);
    Pair p;
    if (k < ho) {
        const double2 yo = fold_dot(Ao + (size_t)k * ho, tile + he * tc, ho, tc, c);
        p.a = make_double2(ye.x + yo.x, ye.y + yo.y);
        p.b = make_double2(ye.x - yo.x, ye.y - yo.y);
    } else {
        p.a = ye;
        p.b = ye;
    }
    return p;
}

__device__ __forceinline__ double2 c2sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// ------------------------------------------------------------------ vorticity
// omega = (wy - vz, uz - wx, vx - uy)  (3D:1077-1079), spectrally.
__device__ __forceinline__ void vorticity_body(GridDev g, Ops ops, const double2* __restrict__ U,
                                               const double2* __restrict__ V,
                                               const double2* __restrict__ W,
                                               double2* __restrict__ OX, double2* __restrict__ OY,
                                               double2* __restrict__ OZ, int tc, int bx) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    double2* tu = sm;
    double2* tv = sm + nz * tc;
    const int m0 = bx * tc;
    fold_load(tu, U, g, m0, tc, he, ho);
    fold_load(tv, V, g, m0, tc, he, ho);
    __syncthreads();
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        const Pair du = anti_apply(ops.D1e, ops.D1o, tu, k, c, tc, he, ho);
        const Pair dv = anti_apply(ops.D1e, ops.D1o, tv, k, c, tc, he, ho);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const int npt = (k < ho) ? 2 : 1;
        for (int p = 0; p < npt; ++p) {
            const int z = p ? nz - 1 - k : k;
            const size_t o = (size_t)z * g.nm + m;
            const double2 w = W[o], u = U[o], v = V[o];
            const double2 wy = i_times(mi.ay, w), wx = i_times(mi.ax, w);
            const double2 vx = i_times(mi.ax, v), uy = i_times(mi.ay, u);
            OX[o] = c2sub(wy, p ? dv.b : dv.a);
            OY[o] = c2sub(p ? du.b : du.a, wx);
            OZ[o] = c2sub(vx, uy);
        }
    }
}

__global__ void __launch_bounds__(256) k_vorticity(GridDev g, Ops ops, const double2* __restrict__ U,
                                                   const double2* __restrict__ V,
                                                   const double2* __restrict__ W,
                                                   double2* __restrict__ OX, double2* __restrict__ OY,
                                                   double2* __restrict__ OZ, int tc) {
    vorticity_body(g, ops, U, V, W, OX, OY, OZ, tc, blockIdx.x);
}

// ------------------------------------------------------------------ products
// S = u x omega (3D:1085-1095) on physical fields: in = u,v,w,ox,oy,oz.
__device__ __forceinline__ void products_body(RFields in, RFields out, size_t n, int bx, int gx) {
    const size_t stride = (size_t)gx * blockDim.x;
    for (size_t i = (size_t)bx * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double u = in.p[0][i], v = in.p[1][i], w = in.p[2][i];
        const double ox = in.p[3][i], oy = in.p[4][i], oz = in.p[5][i];
        out.p[0][i] = v * oz - w * oy;
        out.p[1][i] = w * ox - u * oz;
        out.p[2][i] = u * oy - v * ox;
    }
}

__global__ void k_products(RFields in, RFields out, size_t n) {
    products_body(in, out, n, blockIdx.x, gridDim.x);
}

// Per-mode folded inverse x = G b for the output pair k of column c:
// GT points at [GeT (he x he) | GoT (ho x ho)] stored transposed
// (GeT[j][k] = Ge[k][j]) so that threads of consecutive k read consecutive
// addresses.  bt is the folded rhs tile.
__device__ __forceinline__ Pair inv_apply(const double* __restrict__ GT, const double2* bt, int k, int c, int tc,
                                          int he, int ho) {
    double2 xe = make_double2(0.0, 0.0), xo = xe;
#pragma unroll 4
    for (int j = 0; j < he; ++j) {
        const double gv = __ldg(&GT[(size_t)j * he + k]);
        const double2 b = bt[j * tc + c];
        xe.x = fma(gv, b.x, xe.x);
        xe.y = fma(gv, b.y, xe.y);
    }
    Pair p;
    if (k < ho) {
        const double* __restrict__ GoT = GT + (size_t)he * he;
#pragma unroll 4
        for (int j = 0; j < ho; ++j) {
            const double gv = __ldg(&GoT[(size_t)j * ho + k]);
            const double2 b = bt[(he + j) * tc + c];
            xo.x = fma(gv, b.x, xo.x);
            xo.y = fma(gv, b.y, xo.y);
        }
        p.a = make_double2(xe.x + xo.x, xe.y + xo.y);
        p.b = make_double2(xe.x - xo.x, xe.y - xo.y);
    } else {
        p.a = xe;
        p.b = xe;
    }
    return p;
}

// ------------------------------------------------------------------ viscous step
// viscous_step_3d (3D:1285-1332) + solve_viscous_helmholtz (3D:1425-1521) for
// all three components of a mode tile:
//   R   = F + dt*(mask(S) + dpdx*[comp==u, mode (0,0)]) + cn*(D2.F - k^2 F)
//   b_k = R_k w_k ybar/2,   k interior: b_k -= H(k,1) bc1 + H(k,nz) bc2
//   b_1 = bc1, b_nz = bc2;   F* = A_q^{-1} b   (A_q: rows 1, nz are identity,
//   columns kept, so the wall data enters twice, as in the reference)
// bc: u -> -dt dp/dx|wall, v -> -dt dp/dy|wall (previous total pressure,
// 3D:1325-1326), w -> 0 (3D:1328).
__device__ __forceinline__ double2 viscous_rhs(const GridDev& g, const Ops& ops, const StepParams& sp, int comp,
                                               int z, int m, int ky, int kx, double2 f, double2 s, double2 lap,
                                               double2 bc1, double2 bc2, double dpdx) {
    if (z == 0) return bc1;
    if (z == g.nz - 1) return bc2;
    if (sp.dealias) {  // apply_dealias_truncation (3D:1163-1193)
        const int kyi = ky <= g.ny / 2 ? ky : g.ny - ky;
        if (kx > sp.kx_max || kyi > sp.ky_max) s = make_double2(0.0, 0.0);
    }
    if (comp == 0 && m == 0) s.x += dpdx * sp.forcing_scale;  // 3D:1123-1145
    double2 rr = make_double2(f.x + sp.dt * s.x, f.y + sp.dt * s.y);
    if (sp.cn_fac != 0.0) {  // add_explicit_diffusion (3D:1355-1381)
        const double ksq = __ldg(&ops.ksq[mode_q(ky, kx, g.ny, g.nxhp)]);
        rr.x += sp.cn_fac * (lap.x - ksq * f.x);
        rr.y += sp.cn_fac * (lap.y - ksq * f.y);
    }
    const double whz = __ldg(&ops.wh[z]);
    const double s0 = __ldg(&ops.S0[z]), sn = __ldg(&ops.Sn[z]);
    return make_double2(rr.x * whz - (s0 * bc1.x + sn * bc2.x), rr.y * whz - (s0 * bc1.y + sn * bc2.y));
}

// Crank-Nicolson with the explicit half folded into the solve.  LGL
// quadrature makes the collocation second derivative and the Galerkin
// stiffness agree on interior rows, w_k (D2 f)_k = -(S f)_k (integration by
// parts; the Lagrange basis vanishes at the walls), so with the CN factor
// equal to the implicit one, R_k w_k = 2 w_k f_k - (H f)_k + dt w_k s_k and
//   F*_I = H_II^{-1} r_I - f_I,
//   r_k = w_k (2 f_k + dt s_k) - f S_k1 (f_1 + 2 bc1) - f S_kn (f_nz + 2 bc2),
// the wall data entering twice as in the reference's lifting: one folded
// inverse per component instead of D2 and the inverse.  H_II^{-1} is A_q^{-1}
// applied with zero wall entries.  Wall levels of r are zero.
__device__ __forceinline__ double2 viscous_rhs_cn(const GridDev& g, const Ops& ops, const StepParams& sp, int comp,
                                                  int z, int m, int ky, int kx, double2 f, double2 s, double2 f1,
                                                  double2 fn, double2 bc1, double2 bc2, double dpdx) {
    if (z == 0 || z == g.nz - 1) return make_double2(0.0, 0.0);
    if (sp.dealias) {  // apply_dealias_truncation (3D:1163-1193)
        const int kyi = ky <= g.ny / 2 ? ky : g.ny - ky;
        if (kx > sp.kx_max || kyi > sp.ky_max) s = make_double2(0.0, 0.0);
    }
    if (comp == 0 && m == 0) s.x += dpdx * sp.forcing_scale;  // 3D:1123-1145
    const double whz = __ldg(&ops.wh[z]);
    const double s0 = __ldg(&ops.S0[z]), sn = __ldg(&ops.Sn[z]);
    const double2 l1 = make_double2(f1.x + 2.0 * bc1.x, f1.y + 2.0 * bc1.y);
    const double2 ln = make_double2(fn.x + 2.0 * bc2.x, fn.y + 2.0 * bc2.y);
    return make_double2(whz * (2.0 * f.x + sp.dt * s.x) - (s0 * l1.x + sn * ln.x),
                        whz * (2.0 * f.y + sp.dt * s.y) - (s0 * l1.y + sn * ln.y));
}

// viscous_rhs_cn folded at the level pair (k, nz-1-k), k >= 1, with the
// weights taken out (the tensor-core operator carries 2 w_j G[i][j]): with
// the symmetric weights (w_k = w_nz-1-k) and lifting columns (S0_nz-1-k =
// Sn_k), (r_k + r_k') / (2 w_k) = (a_k + a_k') - tau+_k (l1 + ln) and
// (r_k - r_k') / (2 w_k) = (a_k - a_k') - tau-_k (l1 - ln), with
// a = f + (dt/2) s, the lifting data l1 = f_1 + 2 bc1, ln = f_nz + 2 bc2 and
// tau+-_k = (S0_k +- Sn_k) / (2 w_k) (Ops::tcTau); the unpaired mid level
// (nz odd) gets r_k / (2 w_k) = a_k - (S0_k / 2 w_k)(l1 + ln).  Five FP64
// operations per value instead of the 14 of two viscous_rhs_cn calls and
// their sum and difference.
__device__ __forceinline__ Pair viscous_rhs_cn_half(const GridDev& g, const Ops& ops, const StepParams& sp,
                                                    int comp, int k, int m, int ky, int kx, double2 f1v,
                                                    double2 f2v, double2 s1, double2 s2, double2 l1, double2 ln,
                                                    double dpdx) {
    if (sp.dealias) {  // apply_dealias_truncation (3D:1163-1193)
        const int kyi = ky <= g.ny / 2 ? ky : g.ny - ky;
        if (kx > sp.kx_max || kyi > sp.ky_max) s1 = s2 = make_double2(0.0, 0.0);
    }
    if (comp == 0 && m == 0) {  // 3D:1123-1145
        s1.x += dpdx * sp.forcing_scale;
        s2.x += dpdx * sp.forcing_scale;
    }
    const double hdt = 0.5 * sp.dt;
    const int he = g.nz - g.nz / 2;
    const double tp = __ldg(&ops.tcTau[k]);
    const double2 a1 = make_double2(fma(hdt, s1.x, f1v.x), fma(hdt, s1.y, f1v.y));
    const double2 lp = make_double2(l1.x + ln.x, l1.y + ln.y);
    Pair r;
    if (k < g.nz / 2) {
        const double tm = __ldg(&ops.tcTau[he + k]);
        const double2 a2 = make_double2(fma(hdt, s2.x, f2v.x), fma(hdt, s2.y, f2v.y));
        const double2 lm = make_double2(l1.x - ln.x, l1.y - ln.y);
        r.a = make_double2(fma(-tp, lp.x, a1.x + a2.x), fma(-tp, lp.y, a1.y + a2.y));
        r.b = make_double2(fma(-tm, lm.x, a1.x - a2.x), fma(-tm, lm.y, a1.y - a2.y));
    } else {
        r.a = make_double2(fma(-tp, lp.x, a1.x), fma(-tp, lp.y, a1.y));
        r.b = make_double2(0.0, 0.0);
    }
    return r;
}

// x_I - f_I at an interior level, the wall value at the walls
__device__ __forceinline__ double2 viscous_out_cn(const GridDev& g, int z, double2 x, double2 f, double2 bc1,
                                                  double2 bc2) {
    if (z == 0) return bc1;
    if (z == g.nz - 1) return bc2;
    return make_double2(x.x - f.x, x.y - f.y);
}

__device__ __forceinline__ double2 to_d2(double2 a) { return a; }
__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2((double)a.x, (double)a.y); }

template <typename SrcC>
__device__ __forceinline__ void viscous_body(GridDev g, Ops ops, StepParams sp, Fields F,
                                             FieldsT<SrcC> Src, const double2* __restrict__ GP,
                                             const dns3d_pi_state* __restrict__ pi, Fields Out,
                                             int tc, int bx) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    const int tsz = nz * tc;
    double2* tf = sm;             // [3] folded F tiles
    double2* tb = sm + 3 * tsz;   // [3] folded rhs tiles
    const int m0 = bx * tc;
    const bool cn_id = sp.cn_identity && !sp.rhs_only;
    if (!cn_id)
        for (int comp = 0; comp < 3; ++comp) fold_load(tf + comp * tsz, fptr(F, comp), g, m0, tc, he, ho);
    __syncthreads();
    const double dpdx = pi->current_pressure_gradient;
    if (cn_id) {
        for (int t = threadIdx.x; t < 3 * he * tc; t += blockDim.x) {
            const int comp = t / (he * tc);
            const int r = t - comp * he * tc;
            const int k = r / tc, c = r - k * tc;
            const int m = m0 + c;
            double2* bt = tb + comp * tsz;
            if (m >= g.nm) {
                bt[k * tc + c] = make_double2(0.0, 0.0);
                if (k < ho) bt[(he + k) * tc + c] = make_double2(0.0, 0.0);
                continue;
            }
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            double2 bc1 = make_double2(0.0, 0.0), bc2 = bc1;
            if (comp < 2) {
                const double2 g1 = GP[(size_t)(2 * comp) * g.nm + m];
                const double2 g2 = GP[(size_t)(2 * comp + 1) * g.nm + m];
                bc1 = make_double2(-sp.dt * g1.x, -sp.dt * g1.y);
                bc2 = make_double2(-sp.dt * g2.x, -sp.dt * g2.y);
            }
            const double2* fc = fptr(F, comp);
            const double2 f1 = fc[m], fn = fc[(size_t)(nz - 1) * g.nm + m];
            const int z1 = k, z2 = nz - 1 - k;
            const size_t o1 = (size_t)z1 * g.nm + m, o2 = (size_t)z2 * g.nm + m;
            const double2 b1 = viscous_rhs_cn(g, ops, sp, comp, z1, m, ky, kx, fc[o1],
                                              to_d2(fptr(Src, comp)[o1]), f1, fn, bc1, bc2, dpdx);
            if (k < ho) {
                const double2 b2 = viscous_rhs_cn(g, ops, sp, comp, z2, m, ky, kx, fc[o2],
                                                  to_d2(fptr(Src, comp)[o2]), f1, fn, bc1, bc2, dpdx);
                bt[k * tc + c] = make_double2(b1.x + b2.x, b1.y + b2.y);
                bt[(he + k) * tc + c] = make_double2(b1.x - b2.x, b1.y - b2.y);
            } else {
                bt[k * tc + c] = b1;
            }
        }
        __syncthreads();
        const size_t qs = (size_t)he * he + (size_t)ho * ho;
        // one output pair (k, nz-1-k) of one component per thread
        for (int t = threadIdx.x; t < 3 * he * tc; t += blockDim.x) {
            const int comp = t / (he * tc);
            const int r = t - comp * he * tc;
            const int c = r / he, k = r - c * he;
            const int m = m0 + c;
            if (m >= g.nm) continue;
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            const double* __restrict__ GT = ops.HinvF + (size_t)mode_q(ky, kx, g.ny, g.nxhp) * qs;
            const Pair x = inv_apply(GT, tb + comp * tsz, k, c, tc, he, ho);
            double2 bc1 = make_double2(0.0, 0.0), bc2 = bc1;
            if (comp < 2 && k == 0) {
                const double2 g1 = GP[(size_t)(2 * comp) * g.nm + m];
                const double2 g2 = GP[(size_t)(2 * comp + 1) * g.nm + m];
                bc1 = make_double2(-sp.dt * g1.x, -sp.dt * g1.y);
                bc2 = make_double2(-sp.dt * g2.x, -sp.dt * g2.y);
            }
            const double2* fc = fptr(F, comp);
            double2* oc = fptr(Out, comp);
            const size_t o1 = (size_t)k * g.nm + m;
            oc[o1] = viscous_out_cn(g, k, x.a, fc[o1], bc1, bc2);
            if (k < ho) {
                const size_t o2 = (size_t)(nz - 1 - k) * g.nm + m;
                oc[o2] = viscous_out_cn(g, nz - 1 - k, x.b, fc[o2], bc1, bc2);
            }
        }
        return;
    }
    for (int t = threadIdx.x; t < 3 * he * tc; t += blockDim.x) {
        const int comp = t / (he * tc);
        const int r = t - comp * he * tc;
        const int k = r / tc, c = r - k * tc;
        const int m = m0 + c;
        double2* bt = tb + comp * tsz;
        if (m >= g.nm) {
            bt[k * tc + c] = make_double2(0.0, 0.0);
            if (k < ho) bt[(he + k) * tc + c] = make_double2(0.0, 0.0);
            continue;
        }
        const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
        double2 bc1 = make_double2(0.0, 0.0), bc2 = bc1;
        if (comp < 2) {
            const double2 g1 = GP[(size_t)(2 * comp) * g.nm + m];
            const double2 g2 = GP[(size_t)(2 * comp + 1) * g.nm + m];
            bc1 = make_double2(-sp.dt * g1.x, -sp.dt * g1.y);
            bc2 = make_double2(-sp.dt * g2.x, -sp.dt * g2.y);
        }
        Pair lap;
        lap.a = lap.b = make_double2(0.0, 0.0);
        if (sp.cn_fac != 0.0) lap = sym_apply(ops.D2e, ops.D2o, tf + comp * tsz, k, c, tc, he, ho);
        const int z1 = k, z2 = nz - 1 - k;
        const size_t o1 = (size_t)z1 * g.nm + m, o2 = (size_t)z2 * g.nm + m;
        const double2 b1 = viscous_rhs(g, ops, sp, comp, z1, m, ky, kx, fptr(F, comp)[o1], to_d2(fptr(Src, comp)[o1]),
                                       lap.a, bc1, bc2, dpdx);
        if (k < ho) {
            const double2 b2 = viscous_rhs(g, ops, sp, comp, z2, m, ky, kx, fptr(F, comp)[o2],
                                           to_d2(fptr(Src, comp)[o2]), lap.b, bc1, bc2, dpdx);
            if (sp.rhs_only) fptr(Out, comp)[o2] = b2;
            bt[k * tc + c] = make_double2(b1.x + b2.x, b1.y + b2.y);
            bt[(he + k) * tc + c] = make_double2(b1.x - b2.x, b1.y - b2.y);
        } else {
            bt[k * tc + c] = b1;
        }
        if (sp.rhs_only) fptr(Out, comp)[o1] = b1;
    }
    if (sp.rhs_only) return;  // uniform over the block
    __syncthreads();
    const size_t qstride = (size_t)he * he + (size_t)ho * ho;
    if (tc == 1) {  // a single mode (the mixed form's (0,0) launch): components in parallel
        for (int t = threadIdx.x; t < 3 * he; t += blockDim.x) {
            const int comp = t / he, k = t - comp * he;
            const int m = m0;
            if (m >= g.nm) continue;
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            const double* __restrict__ GT = ops.HinvF + (size_t)mode_q(ky, kx, g.ny, g.nxhp) * qstride;
            const Pair x = inv_apply(GT, tb + comp * tsz, k, 0, 1, he, ho);
            fptr(Out, comp)[(size_t)k * g.nm + m] = x.a;
            if (k < ho) fptr(Out, comp)[(size_t)(nz - 1 - k) * g.nm + m] = x.b;
        }
        return;
    }
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int c = t / he, k = t - c * he;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
        const double* __restrict__ GT = ops.HinvF + (size_t)mode_q(ky, kx, g.ny, g.nxhp) * qstride;
        for (int comp = 0; comp < 3; ++comp) {
            const Pair x = inv_apply(GT, tb + comp * tsz, k, c, tc, he, ho);
            fptr(Out, comp)[(size_t)k * g.nm + m] = x.a;
            if (k < ho) fptr(Out, comp)[(size_t)(nz - 1 - k) * g.nm + m] = x.b;
        }
    }
}

// ------------------------------------------------------------------ tensor-core viscous step
// The Crank-Nicolson viscous step of viscous_body with the folded inverses
// applied on the tensor cores in emulated FP64 (tc.cuh).  A CTA takes qpb
// operator indices q; the modes sharing q ((ky, kx) and (ny-ky, kx)) and
// their three components give 12 right-hand-side columns (re, im), one block
// of 16.  Per q:
//  (a) the lanes of the last warp start bulk copies of the operator's digit
//      slices into blocks E (Ge) and O (Go) of each slice (the K padding stays
//      zero);
//  (b) the weight-free folded right-hand sides are formed in FP64
//      (viscous_rhs_cn_half; the operator carries 2 w_j) from the q's inputs
//      staged in shared memory: the 2 x 3 columns of u, v, w and of the
//      sources, the wall gradients and the row exponents, copied with
//      cp.async while earlier work runs, so the strided column reads (one
//      16-byte value per level, a plane apart) are off the critical path;
//      each column's power-of-two scale comes from the largest key (tc_key)
//      of its values, a warp reduction and one shared atomic per column and
//      warp;
//  (d) the digits, two K rows of one column per thread (tc_digit_pairs);
//  (e) one thread for block E (even rows: right-hand-side rows [0, ke)) and
//      one of the next warp for block O (odd rows: [ke, kt)) issue, per
//      digit slice sa of the operator, the block's K-steps against
//      right-hand-side digit slices 0 .. 7-sa side by side (N = 16 (8-sa)),
//      accumulated into the weight-class columns sa .. 7 of that block's
//      TMEM region;
//  (f) every row's 8 class accumulators are combined into the 64-bit integer
//      T (tc_combine8);
//  (g) the outputs F* = x - f are formed in integers from T of the even and
//      odd rows (which share an exponent) and written (wall values at the
//      walls).
// Two schedules (viscous_tc_pipelined).  Phased, where two CTAs share an SM:
// per q (a) + (b) | (d) | (e) | (f) | (g), each behind a barrier, the other
// CTA filling the waits.  Pipelined, where one CTA has the SM: while the MMAs
// of q run, one pass of the CTA writes the outputs (g) of q - 1 and forms the
// right-hand sides (b) of q + 1 (item for item in the same shared-memory
// slots: each thread reads its results of q - 1 before it writes its
// right-hand sides of q + 1), and the last warp starts the operator copy (a)
// of q + 1 the moment the MMAs of q complete; then the combination (f) of q
// runs beside the digits (d) of q + 1.  Two barriers per q; the right-hand
// sides and results alternate between two buffers, the column keys rotate
// through three, the staged inputs through two (the wall gradients and row
// exponents, which the outputs still read, through four); the state values
// that (g) subtracts stay in registers from (b), two sets in turn.
// (t - round(f 2^-E)) 2^E: an integer result t at the scale 2^E minus an
// FP64 value f, exactly in integers but for the rounding of f to that scale
// and of the final conversion; falls back to the FP64 difference where f is
// non-finite, far above the scale (f 2^-E >= 2^62) or the integer difference
// would overflow.
__device__ __forceinline__ double tc_sub_scaled(long long t, double f, int E) {
    const long long b = __double_as_longlong(f);
    int ex = (int)((b >> 52) & 0x7FF);
    if (ex == 0x7FF) return i2d_scaled(t, E) - f;
    long long m = b & 0xFFFFFFFFFFFFFLL;
    if (ex == 0) {
        if (m == 0) return i2d_scaled(t, E);
        ex = 1;  // subnormal: no implicit bit
    } else {
        m |= 1LL << 52;
    }
    const int sh = 1075 + E - ex;  // f 2^-E = m 2^-sh
    long long F;
    if (sh >= 63) F = 0;  // |f 2^-E| < 2^-10
    else if (sh > 0) F = (m + (1LL << (sh - 1))) >> sh;
    else if (sh >= -9) F = m << (-sh);
    else return i2d_scaled(t, E) - f;
    if (b < 0) F = -F;
    const long long d = (long long)((unsigned long long)t - (unsigned long long)F);
    if (((t ^ F) & (t ^ d)) < 0) return i2d_scaled(t, E) - f;  // overflow
    return i2d_scaled(d, E);
}

// Combination of one warp's TMEM lanes for 6 right-hand-side columns (H = 0:
// columns 0 .. 5, H = 1: 6 .. 11): the 8 weight-class accumulators of each
// column loaded back to back under one wait and combined in 64-bit integers
// (tc_combine8), stored to sR at the lane's row as the integer T (its bits in
// the FP64 slot; the outputs' scale 2^(e + f - 52) is applied in (g)).  The
// two warps of a lane quadrant take one half each.
template <int H>
__device__ __noinline__ void tc_combine6(uint32_t lanes, double* sR, int m8, int row, bool valid) {
    uint32_t r[kTcClasses * 6];
#pragma unroll
    for (int c = 0; c < kTcClasses; ++c) {
        const uint32_t a = lanes + (uint32_t)(c * kTcN + 6 * H);
        if (H == 0) {
            tc_ld4_nw(a, r + 6 * c);
            tc_ld2_nw(a + 4, r + 6 * c + 4);
        } else {  // each load's first column a multiple of its width
            tc_ld2_nw(a, r + 6 * c);
            tc_ld4_nw(a + 2, r + 6 * c + 2);
        }
    }
    tc_ld_wait(r);
    if (valid) {
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const long long T = tc_combine8(r[j], r[6 + j], r[12 + j], r[18 + j], r[24 + j], r[30 + j], r[36 + j],
                                            r[42 + j]);
            sR[(6 * H + j) * m8 + row] = __longlong_as_double(T);  // the integer result, its bits
        }
    }
}

// Bytes of unused shared memory in front of the digit slices: block O's MMA
// starts 64 rows (8 row groups) before its operand, so that its o8 <= 64
// result rows land in TMEM lanes 64 .. 64 + o8 (lane quadrants 2 and 3) while
// block E's use quadrants 0 and 1 (2 as well at nz = 129), and the
// combination spreads over more warps, each reading only its own quadrant.
// Those 64 rows of the first slice must still lie inside the CTA's shared
// memory; rows an MMA reads there only produce accumulator lanes that are
// never read.
__host__ __device__ inline size_t tc_oshift_pad(const TcBlocks& bl) {
    const long long need = 8LL * bl.kO * 16 - (long long)bl.aE * 2;
    return need > 0 ? (size_t)((need + 127) / 128 * 128) : 0;
}
__host__ __device__ inline size_t viscous_tc_pad(const TcGeom& t) { return tc_oshift_pad(tc_blocks(t, false)); }

// Buffers of the viscous tensor-core kernel's two schedules (below): right-
// hand sides / results kR, column keys kK, staged input columns kP, staged
// wall gradients and row exponents kG.
template <bool kPipe>
struct VtcBufs {
    static constexpr int kR = kPipe ? 2 : 1, kK = kPipe ? 3 : 2, kP = kPipe ? 2 : 1, kG = kPipe ? 4 : 2;
};

// Byte offset of the staged inputs in the viscous tensor-core kernel's shared
// memory: after the digit slices, right-hand-side digits, the right-hand-side
// / result buffers, the column keys, barriers, TMEM address and flags
// (16-byte aligned).
template <bool kPipe>
__host__ __device__ inline size_t viscous_tc_stage_offset(const TcGeom& t) {
    using B = VtcBufs<kPipe>;
    const size_t b = viscous_tc_pad(t) + (size_t)kTcSlices * (tc_blocks(t, false).a + kTcN * t.kt) * sizeof(__half) +
                     (size_t)B::kR * kTcN * t.m8 * sizeof(double) + B::kK * kTcN * sizeof(unsigned) +
                     2 * sizeof(uint64_t) + 16;
    return (b + 15) / 16 * 16;
}

// Dynamic shared memory one CTA may use (the sm_100-family opt-in maximum).
constexpr size_t kTcSmemMax = 227 * 1024;

// Staged inputs: kP buffers of one q's 12 columns of nz values (F and the
// sources of both modes' u, v, w), and kG of the wall pressure gradients of
// both modes (8 values) and the q's m8 row exponents.  Where they do not fit
// beside the operands (the pipelined schedule at nz >= 127, the phased one at
// nz = 129) the kernel reads its inputs from global memory in (b) and (g).
template <bool kPipe>
__host__ __device__ inline size_t viscous_tc_stage_bytes(const TcGeom& t, int nz) {
    using B = VtcBufs<kPipe>;
    return (size_t)(B::kP * 12 * nz + 8 * B::kG) * sizeof(double2) + (size_t)B::kG * t.m8 * sizeof(int);
}

template <bool kPipe>
__host__ __device__ inline bool viscous_tc_staged(const TcGeom& t, int nz) {
    return viscous_tc_stage_offset<kPipe>(t) + viscous_tc_stage_bytes<kPipe>(t, nz) <= kTcSmemMax;
}

template <bool kPipe>
__host__ __device__ inline size_t viscous_tc_smem_nz(int nz) {
    const TcGeom t = tc_geom(nz);
    return viscous_tc_stage_offset<kPipe>(t) + (viscous_tc_staged<kPipe>(t, nz) ? viscous_tc_stage_bytes<kPipe>(t, nz) : 0);
}

// The schedule: phased where two CTAs share an SM (228 KB of shared memory,
// 1 KB of it reserved per CTA), whose phases then fill each other's waits;
// pipelined where one CTA has the SM to itself (nz >= 81).  Measured at
// 128x128x65 (phased): 170 us phased, 174 us pipelined; at 512x384x129: 6.14
// ms phased, 5.33 ms pipelined.
__host__ __device__ inline bool viscous_tc_pipelined(int nz) {
    return 2 * (viscous_tc_smem_nz<false>(nz) + 1024) > 228 * 1024;
}

template <bool kPipe>
__device__ __forceinline__ void viscous_tc_body(const GridDev& g, const Ops& ops, const StepParams& sp,
                                                const Fields& F, const Fields& Src,
                                                const double2* __restrict__ GP,
                                                const dns3d_pi_state* __restrict__ pi, const Fields& Out,
                                                int qpb, int bx, int* err) {
    extern __shared__ __align__(128) unsigned char tcsm[];
    const TcGeom t = tc_geom(g.nz);
    const TcBlocks bl = tc_blocks(t, false);
    const int nz = g.nz, he = t.he, ho = t.ho, m8 = t.m8;
    const int b_halves = kTcN * t.kt;
    __half* sA = reinterpret_cast<__half*>(tcsm + viscous_tc_pad(t));
    __half* sB = sA + kTcSlices * bl.a;
    using Bf = VtcBufs<kPipe>;
    double* sR2 = reinterpret_cast<double*>(sB + kTcSlices * b_halves);  // [kR][kTcN][m8]: rhs, then results
    unsigned* sK3 = reinterpret_cast<unsigned*>(sR2 + Bf::kR * kTcN * m8);  // [kK][kTcN] column keys
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sK3 + Bf::kK * kTcN);      // [0] MMAs done, [1] slices landed
    uint32_t* tbase = reinterpret_cast<uint32_t*>(mbar + 2);
    int* landed = reinterpret_cast<int*>(tbase + 1);  // [2]: the slices of this q arrived, as seen by each issuer
    int* nextc = landed + 2;                          // the slices of the next q were started
    // staged inputs: [kP][F, Src][mode 0, 1][u, v, w][nz levels], then the
    // wall gradients [kG][mode][GP row 0..3] and row exponents [kG][m8]
    double2* sP2 = reinterpret_cast<double2*>(tcsm + viscous_tc_stage_offset<kPipe>(t));
    double2* sGP4 = sP2 + Bf::kP * 12 * nz;
    int* sEq4 = reinterpret_cast<int*>(sGP4 + 8 * Bf::kG);
    // the buffers of the operator index q0 + rel
    auto rslot = [&](int rel) { return sR2 + (size_t)((unsigned)rel % Bf::kR) * kTcN * m8; };
    auto kslot = [&](int rel) { return sK3 + ((unsigned)rel % Bf::kK) * kTcN; };
    auto pslot = [&](int rel) { return sP2 + (size_t)((unsigned)rel % Bf::kP) * 12 * nz; };
    auto gslot = [&](int rel) { return (int)((unsigned)rel % Bf::kG); };
    {
        uint4* z = reinterpret_cast<uint4*>(sA);
        const int n16 = kTcSlices * (bl.a + b_halves) / 8;
        for (int i = threadIdx.x; i < n16; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
        if (threadIdx.x < Bf::kK * kTcN) sK3[threadIdx.x] = 0u;
    }
    if (threadIdx.x < 32) tc_alloc(tbase, 2 * kTcDCols);
    if (threadIdx.x == 0) {
        tc_mbar_init(&mbar[0], 2);  // two commits per q: the E and the O issuer
        tc_mbar_init(&mbar[1]);
    }
    tc_fence_proxy();  // the zeroed operands, before any bulk copy or MMA
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tbase;
    const double dpdx = pi->current_pressure_gradient;
    const int q0 = bx * qpb, q1 = min(q0 + qpb, ops.nq);
    const size_t qh = tc_q_halves(t);
    const int nbe = t.e8 >> 3, nbo = t.o8 >> 3;
    const int ncore = t.ncore_e + t.ncore_o;
    const bool staged = viscous_tc_staged<kPipe>(t, nz);
    const int nitems = 6 * he;  // (b) and (g): (mode, component, level pair)
    struct QInfo {
        int kya, kx, nmode;
    };
    auto qinfo = [&](int q) {
        QInfo r;
        r.kya = q / g.nxhp;
        r.kx = q - r.kya * g.nxhp;
        r.nmode = (r.kya > 0 && 2 * r.kya != g.ny) ? 2 : 1;
        return r;
    };
    // cp.async of the inputs of operator index q (both modes' columns of u, v,
    // w and of the sources; a missing second mode is not read): one warp per
    // column, its lanes over the levels; one commit group per q, empty past
    // the CTA's last q or when the inputs are not staged
    auto stage = [&](int q) {
        if (staged && q < q1) {
            const int rel = q - q0;
            const QInfo qi = qinfo(q);
            double2* sP = pslot(rel);
            const int lane = threadIdx.x & 31;
            for (int r = threadIdx.x >> 5; r < 2 * qi.nmode * 3; r += blockDim.x >> 5) {
                const int comp = r % 3, r2 = r / 3;
                const int mi = r2 % qi.nmode, fld = r2 / qi.nmode;
                const int m = (mi ? g.ny - qi.kya : qi.kya) * g.nxhp + qi.kx;
                const double2* src = (fld ? fptr(Src, comp) : fptr(F, comp)) + m;
                double2* dst = sP + (size_t)((fld * 2 + mi) * 3 + comp) * nz;
                for (int z = lane; z < nz; z += 32) cp_async16(dst + z, src + (size_t)z * g.nm);
            }
            const int j = threadIdx.x, b = gslot(rel);
            if (j < 4 * qi.nmode) {  // the wall gradients GP[4][nm] of the modes
                const int mi = j >> 2, w = j & 3;
                const int m = (mi ? g.ny - qi.kya : qi.kya) * g.nxhp + qi.kx;
                cp_async16(sGP4 + 8 * b + 4 * mi + w, GP + (size_t)w * g.nm + m);
            } else if (j >= 32 && j < 32 + m8 / 4) {  // the row exponents, 4 per copy
                cp_async16(sEq4 + b * m8 + 4 * (j - 32), ops.tcE + (size_t)q * m8 + 4 * (j - 32));
            }
        }
        cp_async_commit();
    };
    // (a) digit slices of the operator of q: per digit, one copy per 8-row
    // group (its nonzero core matrices are contiguous in the compact store and
    // in the K-major block), issued by the lanes of the last warp
    auto copy_op = [&](int q) {
        if ((int)threadIdx.x >= (int)blockDim.x - 32) {
            const int lane = threadIdx.x & 31;
            if (lane == 0) tc_mbar_expect(&mbar[1], (uint32_t)(qh * sizeof(__half)));
            __syncwarp();
            const __half* src = ops.tcA + (size_t)q * qh;
            const int ngrp = nbe + nbo;
            for (int j = lane; j < kTcSlices * ngrp; j += 32) {
                const int s = j / ngrp, gm = j - s * ngrp;
                const __half* ss = src + (size_t)s * ncore * 64;
                __half* ds = sA + s * bl.a;
                if (gm < nbe)
                    tc_bulk_g2s(ds + tc_core_off(gm * 8, 0, bl.kE), ss + (size_t)gm * nbe * 64, nbe * 128, &mbar[1]);
                else
                    tc_bulk_g2s(ds + bl.aE + tc_core_off((gm - nbe) * 8, 0, bl.kO),
                                ss + (size_t)(t.ncore_e + (gm - nbe) * nbo) * 64, nbo * 128, &mbar[1]);
            }
        }
    };
    // (b) item i of q: the folded right-hand sides of column pair 6 mi + 2 comp
    // + (0 re, 1 im) at level pair k into the q's buffer; returns the state
    // values at the two levels (kept for (g)) and the keys of the values
    auto rhs_item = [&](int q, const QInfo& qi, int i, double2& v1o, double2& v2o, unsigned& kre, unsigned& kim) {
        const int rel = q - q0;
        const double2* sP = pslot(rel);
        const double2* sGP = sGP4 + 8 * gslot(rel);
        double* sR = rslot(rel);
        const int mi = i / (3 * he);
        const int r = i - mi * 3 * he;
        const int comp = r / he, k = r - comp * he;
        double2 fe = make_double2(0.0, 0.0), fo = fe;
        if (mi < qi.nmode) {
            const int ky = mi ? g.ny - qi.kya : qi.kya;
            const int m = ky * g.nxhp + qi.kx;
            // the F and source columns of this mode: staged, or read from
            // global memory one level (a plane) apart
            const size_t st = staged ? 1 : (size_t)g.nm;
            const double2* fc = staged ? sP + (size_t)(mi * 3 + comp) * nz : fptr(F, comp) + m;
            const double2* sc = staged ? sP + (size_t)((2 + mi) * 3 + comp) * nz : fptr(Src, comp) + m;
            const double2 f1 = fc[0], fn = fc[(size_t)(nz - 1) * st];
            const double2 v1 = fc[(size_t)k * st], v2 = k < ho ? fc[(size_t)(nz - 1 - k) * st] : v1;
            v1o = v1;
            v2o = v2;
            if (k > 0) {  // the wall rows of r are zero
                // lifting data l = f_wall + 2 bc, bc = -dt dp/dx|wall (u), -dt dp/dy|wall (v), 0 (w)
                double2 l1 = f1, ln = fn;
                if (comp < 2) {
                    const double2 g1 = staged ? sGP[4 * mi + 2 * comp] : GP[(size_t)(2 * comp) * g.nm + m];
                    const double2 g2 = staged ? sGP[4 * mi + 2 * comp + 1] : GP[(size_t)(2 * comp + 1) * g.nm + m];
                    const double m2dt = -2.0 * sp.dt;
                    l1 = make_double2(fma(m2dt, g1.x, f1.x), fma(m2dt, g1.y, f1.y));
                    ln = make_double2(fma(m2dt, g2.x, fn.x), fma(m2dt, g2.y, fn.y));
                }
                const double2 s1 = sc[(size_t)k * st];
                const double2 s2 = k < ho ? sc[(size_t)(nz - 1 - k) * st] : s1;
                const Pair rf = viscous_rhs_cn_half(g, ops, sp, comp, k, m, ky, qi.kx, v1, v2, s1, s2, l1, ln, dpdx);
                fe = rf.a;
                fo = rf.b;
            }
        }
        const int c0 = 6 * mi + 2 * comp;
        sR[c0 * m8 + k] = fe.x;
        sR[(c0 + 1) * m8 + k] = fe.y;
        kre = tc_key(fe.x);
        kim = tc_key(fe.y);
        if (k < ho) {
            sR[c0 * m8 + t.e8 + k] = fo.x;
            sR[(c0 + 1) * m8 + t.e8 + k] = fo.y;
            kre = max(kre, tc_key(fo.x));
            kim = max(kim, tc_key(fo.y));
        }
    };
    // (g) item i of q: F* = x - f at the interior levels, the wall values at
    // the walls: rows k of both blocks share the exponent e_k, so x_k - f_k =
    // (Te + To - F) 2^E and x_nz-1-k - f_nz-1-k = (Te - To - F') 2^E with
    // E = e_k + f_c - 52 and F = round(f 2^-E), exactly in integers but for
    // that one rounding of f and the final conversion; v1, v2: the state
    // values at levels k, nz-1-k (read again from F past the kept items)
    auto out_item = [&](int q, const QInfo& qi, int i, int p, double2 v1, double2 v2) {
        const int rel = q - q0;
        const double2* sGP = sGP4 + 8 * gslot(rel);
        const int* sEq = sEq4 + gslot(rel) * m8;
        const double* sR = rslot(rel);
        const unsigned* sK = kslot(rel);
        const int mi = i / (3 * he);
        const int r = i - mi * 3 * he;
        const int comp = r / he, k = r - comp * he;
        const int ky = mi ? g.ny - qi.kya : qi.kya;
        const int m = ky * g.nxhp + qi.kx;
        const int c0 = 6 * mi + 2 * comp;
        double2* oc = fptr(Out, comp);
        const size_t o1 = (size_t)k * g.nm + m, o2 = (size_t)(nz - 1 - k) * g.nm + m;
        if (k == 0) {
            double2 bc1 = make_double2(0.0, 0.0), bc2 = bc1;
            if (comp < 2) {
                const double2 g1 = staged ? sGP[4 * mi + 2 * comp] : GP[(size_t)(2 * comp) * g.nm + m];
                const double2 g2 = staged ? sGP[4 * mi + 2 * comp + 1] : GP[(size_t)(2 * comp + 1) * g.nm + m];
                bc1 = make_double2(-sp.dt * g1.x, -sp.dt * g1.y);
                bc2 = make_double2(-sp.dt * g2.x, -sp.dt * g2.y);
            }
            oc[o1] = bc1;
            oc[o2] = bc2;
            return;
        }
        if (p >= 2) {
            const double2* fc = fptr(F, comp);
            v1 = fc[o1];
            v2 = k < ho ? fc[o2] : v1;
        }
        const int e = staged ? sEq[k] : __ldg(&ops.tcE[(size_t)q * m8 + k]);
        double o1x, o1y, o2x = 0.0, o2y = 0.0;
        {
            const int E = e + tc_exponent_key(sK[c0]) - 52;
            const long long te = __double_as_longlong(sR[c0 * m8 + k]);
            const long long to = k < ho ? __double_as_longlong(sR[c0 * m8 + t.e8 + k]) : 0;
            o1x = tc_sub_scaled(te + to, v1.x, E);
            if (k < ho) o2x = tc_sub_scaled(te - to, v2.x, E);
        }
        {
            const int E = e + tc_exponent_key(sK[c0 + 1]) - 52;
            const long long te = __double_as_longlong(sR[(c0 + 1) * m8 + k]);
            const long long to = k < ho ? __double_as_longlong(sR[(c0 + 1) * m8 + t.e8 + k]) : 0;
            o1y = tc_sub_scaled(te + to, v1.y, E);
            if (k < ho) o2y = tc_sub_scaled(te - to, v2.y, E);
        }
        oc[o1] = make_double2(o1x, o1y);
        if (k < ho) oc[o2] = make_double2(o2x, o2y);
    };
    // the state values of items p = 0, 1 (i = threadIdx.x + p blockDim.x):
    // kA for the q whose outputs the next pass writes, kB (pipelined) for the
    // one after
    double2 kA1[2], kA2[2], kB1[2], kB2[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) kA1[p] = kA2[p] = kB1[p] = kB2[p] = make_double2(0.0, 0.0);
    // one pass of the CTA: the outputs (g) of qg (if qg >= q0) and the
    // right-hand sides (b) of qb (if qb < q1), item for item, then the column
    // keys of qb: per warp and column a warp maximum and one shared atomic;
    // the pipelined schedule then swaps kA and kB
    auto pass = [&](int qg, int qb) {
        const QInfo ig = qinfo(max(qg, q0)), ib = qinfo(min(qb, q1 - 1));
        const bool dog = qg >= q0, dob = qb < q1;
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int p = 0; p * (int)blockDim.x < nitems; ++p) {
            const int i = threadIdx.x + p * blockDim.x;
            unsigned kre = 0u, kim = 0u;
            if (i < nitems) {
                double2 v1 = make_double2(0.0, 0.0), v2 = v1;
                if (p == 0) {
                    v1 = kA1[0];
                    v2 = kA2[0];
                } else if (p == 1) {
                    v1 = kA1[1];
                    v2 = kA2[1];
                }
                if (dog && i < ig.nmode * 3 * he) out_item(qg, ig, i, p, v1, v2);
                if (dob) {
                    rhs_item(qb, ib, i, v1, v2, kre, kim);
                    if (p == 0) {
                        kA1[0] = v1;
                        kA2[0] = v2;
                    } else if (p == 1) {
                        kA1[1] = v1;
                        kA2[1] = v2;
                    }
                }
            }
            const int ifirst = w * 32 + p * (int)blockDim.x;
            if (dob && ifirst < nitems) {  // uniform over the warp
                const int glast = min(ifirst + 31, nitems - 1) / he;
                const int mygrp = i < nitems ? i / he : -1;
                unsigned* sK = kslot(qb - q0);
                for (int gi = ifirst / he; gi <= glast; ++gi) {  // column pair 2 gi, 2 gi + 1
                    const unsigned re = __reduce_max_sync(0xffffffffu, mygrp == gi ? kre : 0u);
                    const unsigned im = __reduce_max_sync(0xffffffffu, mygrp == gi ? kim : 0u);
                    if (lane == 0) {
                        atomicMax(&sK[2 * gi], re);
                        atomicMax(&sK[2 * gi + 1], im);
                    }
                }
            }
        }
        if (kPipe) {
#pragma unroll
            for (int p = 0; p < 2; ++p) {  // kA <-> kB
                const double2 a1 = kA1[p], a2 = kA2[p];
                kA1[p] = kB1[p];
                kA2[p] = kB2[p];
                kB1[p] = a1;
                kB2[p] = a2;
            }
        }
    };
    // (d) digits of the right-hand sides of q, K rows kk, kk + 1 (kk even) of
    // one column per thread, one half2 per digit slice: even levels at K
    // [0, he), odd ones at K [ke, ke + ho); a warp covers the 4 row pairs of an
    // 8-row group for 8 columns, so its 4-byte stores fall in distinct
    // shared-memory banks but for columns 8 apart (the bank of (n, k) in a
    // core matrix is 4 (n mod 8) + (k mod 8)/2)
    auto digits = [&](int q) {
        const int rel = q - q0;
        const double* sR = rslot(rel);
        const unsigned* sK = kslot(rel);
        for (int i = threadIdx.x; i < 12 * (t.kt / 2); i += blockDim.x) {
            const int kp = i & 3, cc = i >> 2;
            const int c = cc % 12, kk = (cc / 12) * 8 + 2 * kp;
            const int r0 = tc_k_row(t, kk), r1 = tc_k_row(t, kk + 1);
            if (r0 < 0) continue;  // padding K rows: zeroed once at the start, never written
            const int f = tc_exponent_key(sK[c]);
            __half2 h[kTcSlices];
            tc_digit_pairs(tc_fixed(sR[c * m8 + r0], f), r1 < 0 ? 0 : tc_fixed(sR[c * m8 + r1], f), h);
            __half2* dst = reinterpret_cast<__half2*>(sB + tc_core_off(c, kk, t.kt));
#pragma unroll
            for (int s = 0; s < kTcSlices; ++s) dst[s * (b_halves / 2)] = h[s];
        }
    };
    // (e) the digit-pair products of q: block E issued by one thread, block O
    // by one of the next warp (independent TMEM columns; pipelined: the first
    // lanes of the last two warps, which have the fewest items in the pass
    // beside the MMAs), each committing to mbar[0] once the operator's slices
    // landed
    auto issue = [&](uint32_t par) {
        const int ie = kPipe ? (int)blockDim.x - 64 : 0, io = ie + 32;
        if ((int)threadIdx.x == ie || (int)threadIdx.x == io) {
            const bool blkO = (int)threadIdx.x == io;
            const int ld = tc_mbar_wait(&mbar[1], par, 1 << 22) ? 1 : 0;
            landed[blkO ? 1 : 0] = ld;
            if (ld && !ops.tc_stall) {
                // descriptors differ only in their start address (16-byte
                // units in the low field; a K offset of k elements is k/8
                // core matrices of 128 B, i.e. k units): one add per MMA.
                // Block O starts 64 rows (8 row groups) before its operand, so
                // its o8 <= 64 result rows land in TMEM lanes 64 .. 64 + o8
                // (lane quadrants 2 and 3) while block E's use quadrants 0 and 1
                // (2 as well at nz = 129): the combination then spreads over
                // more warps, each reading only its own quadrant
                const uint64_t dA = blkO ? tc_desc(tc_smem_u32(sA + bl.aE) - (uint32_t)(8 * bl.kO * 16), 128,
                                                   (uint32_t)bl.kO * 16)
                                         : tc_desc(tc_smem_u32(sA), 128, (uint32_t)bl.kE * 16);
                const uint64_t dB =
                    tc_desc(tc_smem_u32(sB), 128, (uint32_t)t.kt * 16) + (uint64_t)(blkO ? bl.bO : bl.bE);
                const int nk = (blkO ? bl.kO : bl.kE) / 16;
                const uint32_t d0 = tmem + (blkO ? (uint32_t)kTcDCols : 0u);
                for (int sa = 0; sa < kTcSlices; ++sa) {
                    const uint32_t idesc = tc_idesc(kTcN * (kTcSlices - sa));
                    const uint64_t so = (uint64_t)((sa * bl.a * 2) >> 4);
                    for (int ks = 0; ks < nk; ++ks)
                        tc_mma(d0 + (uint32_t)(sa * kTcN), dA + so + (uint64_t)(16 * ks), dB + (uint64_t)(16 * ks),
                               idesc, (sa > 0 || ks > 0) ? 1u : 0u);
                }
            }
            if (!ops.tc_stall) tc_commit(&mbar[0]);  // also when nothing was issued: the waiters are released
        }
    };
    // (f) combine the accumulators of each row of q into its result buffer:
    // warp w reads TMEM lane quadrant w % 4 (lanes 32 (w % 4) .. +31); block
    // E's rows are lanes 0 .. e8, block O's lanes 64 .. 64 + o8.  A quadrant
    // holding rows of one block splits its 12 columns between its two warps
    // (6 each); one holding rows of both blocks (nz = 129: lanes 64 .. 71 of
    // E) gives each warp one block.
    auto combine = [&](int q) {
        double* sR = rslot(q - q0);
        const int w = threadIdx.x >> 5;
        if (w < 8) {
            const int quad = w & 3, half = w >> 2;
            const bool hasE = 32 * quad < t.e8;
            const bool hasO = quad >= 2 && 32 * quad < 64 + t.o8;
            const int lane = 32 * quad + (threadIdx.x & 31);
            const uint32_t lanes = tmem + ((uint32_t)(32 * quad) << 16);
            if (hasE || hasO) {
                const int blk = (hasE && hasO) ? half : (hasO ? 1 : 0);
                const bool valid = blk ? (lane >= 64 && lane - 64 < t.o8) : lane < t.e8;
                const int row = blk ? t.e8 + (lane - 64) : lane;
                const uint32_t lb = lanes + (uint32_t)(blk * kTcDCols);
                if (hasE && hasO) {
                    tc_combine6<0>(lb, sR, m8, row, valid);
                    tc_combine6<1>(lb, sR, m8, row, valid);
                } else if (half == 0) {
                    tc_combine6<0>(lb, sR, m8, row, valid);
                } else {
                    tc_combine6<1>(lb, sR, m8, row, valid);
                }
            }
        }
    };
    bool ok = true;
    const int mlimit = ops.tc_stall ? 1 << 10 : 1 << 22;
    // a run-out wait: the flag, then a second bounded wait for each of the
    // slices' bulk copies and the MMAs of q (and the slices of q + 1, if
    // started) that may still be in flight, before the shared memory and the
    // TMEM columns they write are released
    auto timed_out = [&](uint32_t par, bool next) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            if (!landed[0] || !landed[1]) tc_mbar_wait(&mbar[1], par, 1 << 22);
            tc_mbar_wait(&mbar[0], par, mlimit);
            if (next) tc_mbar_wait(&mbar[1], par ^ 1u, 1 << 22);
        }
    };
    if (!kPipe) {
        // phased: per q, (a) + (b) | (d) | (e) | (f) | (g), the staged inputs
        // of q + 1 arriving during (d)-(g)
        if (q0 < q1) stage(q0);
        for (int q = q0; q < q1; ++q) {
            const int rel = q - q0;
            const uint32_t par = (uint32_t)(rel & 1);
            cp_async_wait_all();
            __syncthreads();  // this q's staged inputs, from every thread's copies
            copy_op(q);
            pass(q0 - 1, q);
            __syncthreads();
            if (q + 1 < q1) stage(q + 1);  // the staging buffer is free again
            if (threadIdx.x < kTcN) kslot(rel + 1)[threadIdx.x] = 0u;  // (g) of q - 1 read them last
            digits(q);
            tc_fence_proxy();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            issue(par);
            const bool done = __syncthreads_and(tc_mbar_wait(&mbar[0], par, mlimit)) && landed[0] && landed[1];
            tc_fence_after();
            if (!done) {
                timed_out(par, false);
                ok = false;
                break;  // uniform: no TMEM read, no further MMA
            }
            combine(q);
            tc_fence_before();
            __syncthreads();
            pass(q, q1);
            __syncthreads();  // shared buffers are reused by the next q
        }
    } else if (q0 < q1) {
        // pipelined
        stage(q0);
        stage(q0 + 1);
        cp_async_wait_one();  // q0's inputs
        __syncthreads();
        copy_op(q0);
        pass(q0 - 1, q0);
        __syncthreads();  // q0's right-hand sides and column keys; its staging buffer is free
        stage(q0 + 2);
        digits(q0);
        cp_async_wait_one();  // q0 + 1's inputs
        tc_fence_proxy();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        for (int q = q0; q < q1; ++q) {
            const uint32_t par = (uint32_t)((q - q0) & 1);
            issue(par);
            // the last warp: as soon as the slices of q have landed and its
            // MMAs are done, the slices of q + 1 (flagged in *nextc for the
            // timeout path)
            if ((int)threadIdx.x >= (int)blockDim.x - 32) {
                __syncwarp();  // lane 0 has issued its MMAs
                if ((threadIdx.x & 31) == 0) *nextc = 0;
                if (q + 1 < q1) {
                    const bool rdy = tc_mbar_wait(&mbar[1], par, 1 << 22) && tc_mbar_wait(&mbar[0], par, mlimit);
                    if (__all_sync(0xffffffffu, rdy)) {
                        copy_op(q + 1);
                        if ((threadIdx.x & 31) == 0) *nextc = 1;
                    }
                }
            }
            pass(q - 1, q + 1);  // beside the MMAs of q
            const bool done = __syncthreads_and(tc_mbar_wait(&mbar[0], par, mlimit)) && landed[0] && landed[1];
            tc_fence_after();
            if (!done) {
                timed_out(par, *nextc != 0);
                ok = false;
                break;  // uniform: no TMEM read, no further MMA
            }
            stage(q + 3);  // into the buffers (b) of q + 1 and (g) of q - 1 read last
            combine(q);
            if (threadIdx.x < kTcN) kslot(q + 2 - q0)[threadIdx.x] = 0u;  // (g) of q - 1 read them last
            if (q + 1 < q1) digits(q + 1);
            cp_async_wait_one();  // q + 2's inputs
            tc_fence_proxy();
            tc_fence_before();
            __syncthreads();  // results of q, digits of q + 1; TMEM free for the MMAs of q + 1
            tc_fence_after();
        }
        if (ok) pass(q1 - 1, q1);  // the outputs of the last q
    }
    cp_async_wait_all();  // a stage issued before a timeout lands before the CTA leaves
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tc_dealloc(tmem, 2 * kTcDCols);
}

template <bool kPipe>
__global__ void __launch_bounds__(256, 2) k_viscous_tc(GridDev g, Ops ops, StepParams sp, Fields F, Fields Src,
                                                       const double2* __restrict__ GP,
                                                       const dns3d_pi_state* __restrict__ pi, Fields Out, int qpb,
                                                       int* err) {
    viscous_tc_body<kPipe>(g, ops, sp, F, Src, GP, pi, Out, qpb, blockIdx.x, err);
}

// ------------------------------------------------------------------ tensor-core z-derivatives
// The fixed z-derivative D1 (folded, block anti-diagonal [[0, De], [Do, 0]] on
// [fe; fo]) applied to Op::kFields spectral fields as emulated-FP64
// tensor-core products (tc.cuh), then Op::out_level forms the kernel's outputs from
// the derivatives exactly as the FP64-pipe kernel does.  D1 is the same for
// every mode, so its digit image is copied into shared memory once per CTA
// and a CTA runs tiles of kTcVortCols right-hand-side columns (modes x fields
// x re/im; 16, so that two 512-thread CTAs share an SM).
// Per tile: (b) fold the fields; (c) column scales; (d) digits; (e) per digit
// slice sa of D1, the K-steps of block E (De: even outputs from the odd
// inputs; issued by thread 0) and block O (Do: odd outputs from the even
// inputs; thread 32) against the right-hand-side digit slices 0..7-sa side
// by side, N = 16 (8-sa), into 8 weight-class accumulators per block (256
// TMEM columns); (f) int64 combination -> D1.f in FP64; (g) Op::out_level
// per level.
constexpr int kTcVortCols = 16;  // right-hand-side columns per tile (2 CTAs of 512 threads per SM)
constexpr int kTcVortModes = kTcVortCols / 4;  // modes per tile: u, v x re, im
constexpr int kTcCorrModes = kTcVortCols / 2;  // modes per tile: phi x re, im
constexpr int kTcVortThreads = 512;

// Byte offset of the staged input columns in the z-derivative kernels' shared
// memory (after the pad of the shifted block O, the D1 image, digits,
// results, exponents, barriers), and whether they fit (kTcVortCols / 2
// columns of nz values).
__host__ __device__ inline size_t dz_tc_stage_offset(const TcGeom& t) {
    const TcBlocks bl = tc_blocks(t, true);
    const size_t b = tc_oshift_pad(bl) + (size_t)kTcSlices * (bl.a + kTcVortCols * t.kt) * sizeof(__half) +
                     (size_t)kTcVortCols * t.m8 * sizeof(double) + (size_t)(t.m8 + kTcVortCols) * sizeof(int) +
                     2 * sizeof(uint64_t) + 16;
    return (b + 15) / 16 * 16;
}
__host__ __device__ inline bool dz_tc_staged(const TcGeom& t, int nz) {
    return dz_tc_stage_offset(t) + (size_t)(kTcVortCols / 2) * nz * sizeof(double2) <= kTcSmemMax;
}

template <class Op>
__device__ __forceinline__ void dz_tc_body(const GridDev& g, const Ops& ops, const Op& op, int tile0, int tile1,
                                           int* err) {
    constexpr int kModes = kTcVortCols / (2 * Op::kFields);
    extern __shared__ __align__(128) unsigned char tcsm[];
    const TcGeom t = tc_geom(g.nz);
    const TcBlocks bl = tc_blocks(t, true);
    const int nz = g.nz, he = t.he, ho = t.ho, m8 = t.m8;
    const int b_halves = kTcVortCols * t.kt;
    __half* sA = reinterpret_cast<__half*>(tcsm + tc_oshift_pad(bl));
    __half* sB = sA + kTcSlices * bl.a;
    double* sR = reinterpret_cast<double*>(sB + kTcSlices * b_halves);  // [32][m8]: folded u, v, then D1.u, D1.v
    int* sE = reinterpret_cast<int*>(sR + kTcVortCols * m8);            // row exponents of D1
    int* sF = sE + m8;                                                  // column exponents
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sF + kTcVortCols);     // [0] MMAs done, [1] D1 landed
    uint32_t* tbase = reinterpret_cast<uint32_t*>(mbar + 2);
    int* landed = reinterpret_cast<int*>(tbase + 1);  // [2]: the D1 image arrived, as seen by each issuer
    // staged input columns of one tile: [mode][field][nz]
    double2* sP = reinterpret_cast<double2*>(tcsm + dz_tc_stage_offset(t));
    const bool staged = dz_tc_staged(t, nz);
    const int tid = threadIdx.x;
    {
        uint4* z = reinterpret_cast<uint4*>(sB);
        for (int i = tid; i < kTcSlices * b_halves / 8; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    for (int i = tid; i < m8; i += blockDim.x) sE[i] = __ldg(&ops.tcDE[i]);
    if (tid < 32) tc_alloc(tbase, 2 * kTcClasses * kTcVortCols);
    if (tid == 0) {
        tc_mbar_init(&mbar[0], 2);  // two commits per tile: the E and the O issuer
        tc_mbar_init(&mbar[1]);
        landed[0] = landed[1] = 0;
    }
    tc_fence_proxy();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tbase;
    if (tid == 0) {  // the D1 digit image, once
        tc_mbar_expect(&mbar[1], (uint32_t)(kTcSlices * bl.a * sizeof(__half)));
        for (int s = 0; s < kTcSlices; ++s)
            tc_bulk_g2s(sA + s * bl.a, ops.tcD + (size_t)s * bl.a, (uint32_t)(bl.a * sizeof(__half)), &mbar[1]);
    }
    const int nv = he + ho;
    // cp.async of a tile's input columns into sP, while the tile before it
    // runs its digits, products and outputs
    auto stage = [&](int tile) {
        if (!staged) return;
        const int m0 = tile * kModes;
        // the tile's modes fastest: adjacent lanes copy adjacent modes of one level
        for (int j = tid; j < kModes * Op::kFields * nz; j += blockDim.x) {
            const int mi = j % kModes, r = j / kModes;
            const int f = r % Op::kFields, z = r / Op::kFields;
            if (m0 + mi < g.nm)
                cp_async16(sP + (size_t)(mi * Op::kFields + f) * nz + z, op.field(f) + (size_t)z * g.nm + m0 + mi);
        }
        cp_async_commit();
    };
    if (tile0 < tile1) stage(tile0);
    for (int tile = tile0; tile < tile1; ++tile) {
        const uint32_t par = (uint32_t)((tile - tile0) & 1);
        const int m0 = tile * kModes;
        cp_async_wait_all();
        __syncthreads();  // this tile's staged columns, from every thread's copies
        // (b) folded fields: column 2 (kFields mi + f) + (0 re, 1 im)
        for (int i = tid; i < Op::kFields * kModes * he; i += blockDim.x) {
            const int mi = i / (Op::kFields * he);
            const int r = i - mi * Op::kFields * he;
            const int f = r / he, k = r - f * he;
            const int m = m0 + mi;
            double2 a = make_double2(0.0, 0.0), b = a;
            if (m < g.nm) {
                if (staged) {
                    const double2* col = sP + (size_t)(mi * Op::kFields + f) * nz;
                    a = col[k];
                    if (k < ho) b = col[nz - 1 - k];
                } else {
                    const double2* src = op.field(f);
                    a = src[(size_t)k * g.nm + m];
                    if (k < ho) b = src[(size_t)(nz - 1 - k) * g.nm + m];
                }
            }
            const int c0 = 2 * (Op::kFields * mi + f);
            if (k < ho) {
                sR[c0 * m8 + k] = a.x + b.x;
                sR[(c0 + 1) * m8 + k] = a.y + b.y;
                sR[c0 * m8 + t.e8 + k] = a.x - b.x;
                sR[(c0 + 1) * m8 + t.e8 + k] = a.y - b.y;
            } else {
                sR[c0 * m8 + k] = a.x;
                sR[(c0 + 1) * m8 + k] = a.y;
            }
        }
        __syncthreads();
        if (tile + 1 < tile1) stage(tile + 1);  // sP is free again
        // (c) column scales
        {
            const int w = tid >> 5, l = tid & 31;
            for (int c = w; c < kTcVortCols; c += blockDim.x >> 5) {
                unsigned long long mx = 0;
                for (int k = l; k < nv; k += 32) {
                    const int row = k < he ? k : t.e8 + (k - he);
                    const unsigned long long ab =
                        (unsigned long long)__double_as_longlong(sR[c * m8 + row]) & 0x7FFFFFFFFFFFFFFFULL;
                    mx = ab > mx ? ab : mx;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
                    mx = v > mx ? v : mx;
                }
                if (l == 0) sF[c] = tc_exponent(mx);
            }
        }
        __syncthreads();
        // (d) digits, K rows kk, kk + 1 (kk even) of one column per thread
        // (a warp: the 4 row pairs of an 8-row group for 8 columns, distinct
        // banks): even levels at K [0, he), odd ones at K [ke, ke + ho)
        for (int i = tid; i < kTcVortCols * (t.kt / 2); i += blockDim.x) {
            const int kp = i & 3, cc = i >> 2;
            const int c = cc % kTcVortCols, kk = (cc / kTcVortCols) * 8 + 2 * kp;
            const int r0 = tc_k_row(t, kk), r1 = tc_k_row(t, kk + 1);
            if (r0 < 0) continue;  // padding K rows: zeroed once at the start, never written
            __half2 h[kTcSlices];
            tc_digit_pairs(tc_fixed(sR[c * m8 + r0], sF[c]), r1 < 0 ? 0 : tc_fixed(sR[c * m8 + r1], sF[c]), h);
            __half2* dst = reinterpret_cast<__half2*>(sB + tc_core_off(c, kk, t.kt));
#pragma unroll
            for (int s = 0; s < kTcSlices; ++s) dst[s * (b_halves / 2)] = h[s];
        }
        tc_fence_proxy();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // (e) the digit-pair products: block E issued by thread 0, block O by
        // thread 32 (independent TMEM columns), each committing to mbar[0]
        if (tid == 0 || tid == 32) {
            const bool blkO = tid == 32;
            int ld = landed[blkO ? 1 : 0];
            if (tile == tile0) {
                ld = tc_mbar_wait(&mbar[1], 0, 1 << 22) ? 1 : 0;
                landed[blkO ? 1 : 0] = ld;
            }
            if (ld && !ops.tc_stall) {
                // the descriptors differ only in their start address (16-byte
                // units; a K offset of k elements is k units): one add per MMA.
                // Block O starts 64 rows before its operand: its results land in
                // TMEM lanes 64 .. 64 + o8 (tc_oshift_pad)
                const uint64_t dA = blkO ? tc_desc(tc_smem_u32(sA + bl.aE) - (uint32_t)(8 * bl.kO * 16), 128,
                                                   (uint32_t)bl.kO * 16)
                                         : tc_desc(tc_smem_u32(sA), 128, (uint32_t)bl.kE * 16);
                const uint64_t dB = tc_desc(tc_smem_u32(sB), 128, (uint32_t)t.kt * 16) + (uint64_t)(blkO ? bl.bO : bl.bE);
                const int nk = (blkO ? bl.kO : bl.kE) / 16;
                const uint32_t d0 = tmem + (blkO ? (uint32_t)(kTcClasses * kTcVortCols) : 0u);
                for (int sa = 0; sa < kTcSlices; ++sa) {
                    const uint32_t idesc = tc_idesc(kTcVortCols * (kTcSlices - sa));
                    const uint64_t so = (uint64_t)((sa * bl.a * 2) >> 4);
                    for (int ks = 0; ks < nk; ++ks)
                        tc_mma(d0 + (uint32_t)(sa * kTcVortCols), dA + so + (uint64_t)(16 * ks), dB + (uint64_t)(16 * ks),
                               idesc, (sa > 0 || ks > 0) ? 1u : 0u);
                }
            }
            if (!ops.tc_stall) tc_commit(&mbar[0]);
        }
        // (f) combination: warps w and w + 4k share TMEM lane quadrant w % 4;
        // warp group w / 4 takes every ngrp-th block of 8 of the 32 columns
        const bool done =
            __syncthreads_and(tc_mbar_wait(&mbar[0], par, ops.tc_stall ? 1 << 10 : 1 << 22)) && landed[0] && landed[1];
        tc_fence_after();
        if (!done) {
            if (tid == 0) {
                atomicExch(err, 1);
                // second bounded waits for copies and MMAs still in flight
                // (as in viscous_tc_body) before shared memory and TMEM go
                if (!landed[0] || !landed[1]) tc_mbar_wait(&mbar[1], 0, 1 << 22);
                tc_mbar_wait(&mbar[0], par, ops.tc_stall ? 1 << 10 : 1 << 22);
            }
            break;
        }
        {
            // warp w reads TMEM lane quadrant w % 4: block E's rows are lanes
            // 0 .. e8, block O's lanes 64 .. 64 + o8; the warps of a quadrant
            // (w / 4 = 0 .. 3) take its (block, 4-column group) items, each
            // item's 8 class accumulators loaded back to back under one wait
            constexpr int kGroups = kTcVortCols / 4;
            const int w = tid >> 5, quad = w & 3, grp = w >> 2, ngrp = (int)(blockDim.x >> 7);
            const int lane = 32 * quad + (tid & 31);
            const bool hasE = 32 * quad < t.e8;
            const bool hasO = quad >= 2 && 32 * quad < 64 + t.o8;
            const int nitems = ((int)hasE + (int)hasO) * kGroups;
            for (int it = grp; it < nitems; it += ngrp) {
                const int blk = (hasE && it < kGroups) ? 0 : 1, cb = it % kGroups;
                const uint32_t base = tmem + ((uint32_t)(32 * quad) << 16) +
                                      (uint32_t)(blk * kTcClasses * kTcVortCols + 4 * cb);
                uint32_t r[4 * kTcClasses];
#pragma unroll
                for (int c = 0; c < kTcClasses; ++c) tc_ld4_nw(base + (uint32_t)(c * kTcVortCols), r + 4 * c);
                tc_ld_wait(r);
                const bool valid = blk ? (lane >= 64 && lane - 64 < t.o8) : lane < t.e8;
                if (valid) {
                    const int row = blk ? t.e8 + (lane - 64) : lane;
                    const int e = sE[row];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int col = 4 * cb + j;
                        const long long T = tc_combine8(r[j], r[4 + j], r[8 + j], r[12 + j], r[16 + j], r[20 + j],
                                                        r[24 + j], r[28 + j]);
                        sR[col * m8 + row] = i2d_scaled(T, e + sF[col] - 52);
                    }
                }
            }
        }
        tc_fence_before();
        __syncthreads();
        // (g) the outputs: one level z of one mode per item when the tile's
        // levels fit one pass of the CTA (z and its mirror nz-1-z share the
        // folded row k: ye + yo below the middle, ye - yo above), else one
        // level pair per item; the tile's modes fastest, so adjacent lanes
        // read and write adjacent modes of one level (kModes x 16 bytes)
        const bool per_level = kModes * nz <= (int)blockDim.x;
        const int nlev = per_level ? nz : he;
        for (int i = tid; i < kModes * nlev; i += blockDim.x) {
            const int mi = i % kModes, zi = i / kModes;
            const int m = m0 + mi;
            if (m >= g.nm) continue;
            const int k = (per_level && zi >= he) ? nz - 1 - zi : zi;
            // D1.f at level k (upper = false) or nz-1-k (upper = true)
            auto level = [&](bool upper, double2* d) {
#pragma unroll
                for (int f = 0; f < Op::kFields; ++f) {
                    const int c0 = 2 * (Op::kFields * mi + f);
                    const double2 ye = make_double2(sR[c0 * m8 + k], sR[(c0 + 1) * m8 + k]);
                    const double2 yo = k < ho ? make_double2(sR[c0 * m8 + t.e8 + k], sR[(c0 + 1) * m8 + t.e8 + k])
                                              : make_double2(0.0, 0.0);
                    d[f] = upper ? make_double2(ye.x - yo.x, ye.y - yo.y) : make_double2(ye.x + yo.x, ye.y + yo.y);
                }
            };
            double2 d[Op::kFields];
            if (per_level) {
                level(zi >= he, d);
                op.out_level(g, ops, m, zi, d);
            } else {
                level(false, d);
                op.out_level(g, ops, m, k, d);
                if (k < ho) {
                    level(true, d);
                    op.out_level(g, ops, m, nz - 1 - k, d);
                }
            }
        }
        __syncthreads();  // sR and sB are reused by the next tile
    }
    cp_async_wait_all();  // a stage issued before a timeout lands before the CTA leaves
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tc_dealloc(tmem, 2 * kTcClasses * kTcVortCols);
}

// omega = (wy - vz, uz - wx, vx - uy) from D1.u, D1.v, as vorticity_body forms it
struct VortTcOp {
    static constexpr int kFields = 2;
    const double2* __restrict__ U;
    const double2* __restrict__ V;
    const double2* __restrict__ W;
    double2* __restrict__ OX;
    double2* __restrict__ OY;
    double2* __restrict__ OZ;
    __device__ const double2* field(int f) const { return f ? V : U; }
    // the outputs at level z of mode m from d = (D1.u, D1.v) there
    __device__ void out_level(const GridDev& g, const Ops& ops, int m, int z, const double2* d) const {
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const size_t o = (size_t)z * g.nm + m;
        const double2 w = W[o], u = U[o], v = V[o];
        const double2 du = d[0], dv = d[1];
        // (i ay) w - dv, du - (i ax) w, (i ax) v - (i ay) u with fused products
        OX[o] = make_double2(fma(-mi.ay, w.y, -dv.x), fma(mi.ay, w.x, -dv.y));
        OY[o] = make_double2(fma(mi.ax, w.y, du.x), fma(-mi.ax, w.x, du.y));
        OZ[o] = make_double2(fma(-mi.ax, v.y, mi.ay * u.y), fma(mi.ax, v.x, -(mi.ay * u.x)));
    }
};

// u, v, w of the projection at level z into U, V, W[o]; with sp.bc_walls the
// wall planes get apply_boundary_conditions_3d's zeros (3D:1953-1972) in the
// same pass.
__device__ __forceinline__ void store_projection(const StepParams& sp, int z, int nz, size_t o, double2 u,
                                                 double2 v, double2 w, double2* __restrict__ U,
                                                 double2* __restrict__ V, double2* __restrict__ W) {
    if (sp.bc_walls && (z == 0 || z == nz - 1)) u = v = w = make_double2(0.0, 0.0);
    U[o] = u;
    V[o] = v;
    W[o] = w;
}

// pressure_correction_3d from D1.phi, as correction_body forms it
struct CorrTcOp {
    static constexpr int kFields = 1;
    StepParams sp;
    const double2* __restrict__ US;
    const double2* __restrict__ VS;
    const double2* __restrict__ WS;
    const double2* __restrict__ PHI;
    double2* __restrict__ U;
    double2* __restrict__ V;
    double2* __restrict__ W;
    double2* __restrict__ P;
    double2* __restrict__ GP;
    __device__ const double2* field(int) const { return PHI; }
    // the projection at level z of mode m from d = D1.phi there
    __device__ void out_level(const GridDev& g, const Ops& ops, int m, int z, const double2* dd) const {
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const double dt = sp.dt, dax = dt * mi.ax, day = dt * mi.ay;
        const double2 d = dd[0];
        const size_t o = (size_t)z * g.nm + m;
        const double2 ph = PHI[o];
        const double2 us = US[o], vs = VS[o], ws = WS[o];
        // u* - dt (i ax) phi, v* - dt (i ay) phi, w* - dt dphi/dz
        store_projection(sp, z, g.nz, o, make_double2(fma(dax, ph.y, us.x), fma(-dax, ph.x, us.y)),
                         make_double2(fma(day, ph.y, vs.x), fma(-day, ph.x, vs.y)),
                         make_double2(fma(-dt, d.x, ws.x), fma(-dt, d.y, ws.y)), U, V, W);
        double2 pp = P[o];
        pp.x += ph.x;
        pp.y += ph.y;
        P[o] = pp;
        if (z == 0 || z == g.nz - 1) {
            const int wall = (z == 0) ? 0 : 1;
            GP[(size_t)wall * g.nm + m] = i_times(mi.ax, pp);
            GP[(size_t)(2 + wall) * g.nm + m] = i_times(mi.ay, pp);
        }
    }
};

template <class Op>
__global__ void __launch_bounds__(kTcVortThreads, 2) k_dz_tc(GridDev g, Ops ops, Op op, int chunk, int* err) {
    constexpr int kModes = kTcVortCols / (2 * Op::kFields);
    const int ntiles = (g.nm + kModes - 1) / kModes;
    const int t0 = blockIdx.x * chunk;
    dz_tc_body(g, ops, op, t0, min(t0 + chunk, ntiles), err);
}

template <typename SrcC>
__global__ void __launch_bounds__(256) k_viscous(GridDev g, Ops ops, StepParams sp, Fields F,
                                                 FieldsT<SrcC> Src, const double2* __restrict__ GP,
                                                 const dns3d_pi_state* __restrict__ pi, Fields Out,
                                                 int tc) {
    viscous_body<SrcC>(g, ops, sp, F, Src, GP, pi, Out, tc, blockIdx.x);
}

// ------------------------------------------------------------------ pressure
// solve_pressure_3d_standard (3D:1654-1733): b = (DX u* + DY v* + Dz w*)/dt *
// w ybar/2; or _weak_form (3D:1749-1835): b = (-(DX u* + DY v*) w ybar/2 -
// sum_m d1(m,k) w*_m zwts_m (2/ybar)) / dt.  Mode (0,0): b_1 = 0 and the
// pinned operator (3D:1702-1711), which is not centro-symmetric and is applied
// unfolded.  phi = P_q^{-1} b.
__device__ __forceinline__ double2 pressure_rhs(const GridDev& g, const Ops& ops, const StepParams& sp, int z,
                                                int m, const ModeInfo& mi, const double2* __restrict__ US,
                                                const double2* __restrict__ VS, double2 dz) {
    const size_t o = (size_t)z * g.nm + m;
    const double2 hx = i_times(mi.ax, US[o]);
    const double2 hy = i_times(mi.ay, VS[o]);
    const double whz = __ldg(&ops.wh[z]);
    const double inv_dt = sp.inv_dt;
    double2 b;
    if (!sp.weak_form) {
        b.x = ((hx.x + hy.x) + dz.x) * inv_dt * whz;
        b.y = ((hx.y + hy.y) + dz.y) * inv_dt * whz;
    } else {
        b.x = (-(hx.x + hy.x) * whz - dz.x) * inv_dt;
        b.y = (-(hx.y + hy.y) * whz - dz.y) * inv_dt;
    }
    if (m == 0 && z == 0) b = make_double2(0.0, 0.0);
    return b;
}

// Residual of the Galerkin Poisson system the pressure step solves
// (solve_pressure_3d_standard, DNS_pressure_BC_3D.f90:1680-1714, or the weak
// form 1793-1816): r = b(u*) - P phi with P = -S - diag(k^2 w ybar/2), the
// right-hand side b formed from u*, v*, w* exactly as the FP64 pressure
// kernel forms it, and phi the solution the step left in PHI; mode (0,0)
// without its pinned row and column.  Every row is an equation of the system
// (the Neumann problem has no boundary rows).  Per CTA a tile of tc modes;
// max |r| and max |b| (over re and im parts) go to out[0], out[1] as the bits
// of non-negative doubles (atomicMax on their bit patterns).
__global__ void __launch_bounds__(256) k_poisson_residual(GridDev g, Ops ops, StepParams sp,
                                                          const double2* __restrict__ US,
                                                          const double2* __restrict__ VS,
                                                          const double2* __restrict__ WS,
                                                          const double2* __restrict__ PHI, int tc,
                                                          unsigned long long* out) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    double2* tw = sm;                 // folded w* tile [nz][tc]
    double2* tp = sm + (size_t)nz * tc;  // phi tile, unfolded [nz][tc]
    const int m0 = blockIdx.x * tc;
    fold_load(tw, WS, g, m0, tc, he, ho);
    for (int t = threadIdx.x; t < nz * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        tp[t] = m < g.nm ? PHI[(size_t)k * g.nm + m] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const double* __restrict__ Ae = sp.weak_form ? ops.W1e : ops.D1e;
    const double* __restrict__ Ao = sp.weak_form ? ops.W1o : ops.D1o;
    double rmax = 0.0, bmax = 0.0;
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        const Pair dz = anti_apply(Ae, Ao, tw, k, c, tc, he, ho);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const int q = mode_q(mi.ky, mi.kx, g.ny, g.nxhp);
        const double k2 = __ldg(&ops.ksq[q]);
        for (int h = 0; h < (k < ho ? 2 : 1); ++h) {
            const int z = h ? nz - 1 - k : k;
            if (m == 0 && z == 0) continue;  // the pinned row
            const double2 b = pressure_rhs(g, ops, sp, z, m, mi, US, VS, h ? dz.b : dz.a);
            double2 sp_ = make_double2(0.0, 0.0);  // (S phi)_z over the columns kept
            for (int n = (m == 0 ? 1 : 0); n < nz; ++n) {
                const double a = __ldg(&ops.S[(size_t)z * nz + n]);
                const double2 f = tp[n * tc + c];
                sp_.x = fma(a, f.x, sp_.x);
                sp_.y = fma(a, f.y, sp_.y);
            }
            const double2 f = tp[z * tc + c];
            const double kw = k2 * __ldg(&ops.wh[z]);
            const double rx = b.x + sp_.x + kw * f.x, ry = b.y + sp_.y + kw * f.y;
            rmax = fmax(rmax, fmax(fabs(rx), fabs(ry)));
            bmax = fmax(bmax, fmax(fabs(b.x), fabs(b.y)));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(rmax));
        atomicMax(&out[1], (unsigned long long)__double_as_longlong(bmax));
    }
}

__device__ __forceinline__ void pressure_body(GridDev g, Ops ops, StepParams sp,
                                              const double2* __restrict__ US,
                                              const double2* __restrict__ VS,
                                              const double2* __restrict__ WS,
                                              double2* __restrict__ PHI, int tc, int bx) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    const int tsz = nz * tc;
    double2* tw = sm;            // folded w* tile
    double2* tb = sm + tsz;      // folded rhs tile
    double2* bpin = sm + 2 * tsz;  // unfolded rhs of mode (0,0)
    const int m0 = bx * tc;
    fold_load(tw, WS, g, m0, tc, he, ho);
    __syncthreads();
    const double* __restrict__ Ae = sp.weak_form ? ops.W1e : ops.D1e;
    const double* __restrict__ Ao = sp.weak_form ? ops.W1o : ops.D1o;
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) {
            tb[t] = make_double2(0.0, 0.0);
            if (k < ho) tb[(he + k) * tc + c] = make_double2(0.0, 0.0);
            continue;
        }
        const Pair dz = anti_apply(Ae, Ao, tw, k, c, tc, he, ho);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const double2 b1 = pressure_rhs(g, ops, sp, k, m, mi, US, VS, dz.a);
        if (k < ho) {
            const double2 b2 = pressure_rhs(g, ops, sp, nz - 1 - k, m, mi, US, VS, dz.b);
            tb[t] = make_double2(b1.x + b2.x, b1.y + b2.y);
            tb[(he + k) * tc + c] = make_double2(b1.x - b2.x, b1.y - b2.y);
            if (m == 0) { bpin[k] = b1; bpin[nz - 1 - k] = b2; }
            if (sp.rhs_only && m != 0) PHI[(size_t)(nz - 1 - k) * g.nm + m] = b2;
        } else {
            tb[t] = b1;
            if (m == 0) bpin[k] = b1;
        }
        if (sp.rhs_only && m != 0) PHI[(size_t)k * g.nm + m] = b1;
    }
    __syncthreads();
    const size_t qstride = (size_t)he * he + (size_t)ho * ho;
    if (tc == 1 && m0 == 0) {  // the pinned mode alone (the mixed form's launch): one output level per thread
        for (int z = threadIdx.x; z < nz; z += blockDim.x) {
            double2 a = make_double2(0.0, 0.0);
#pragma unroll 4
            for (int zp = 0; zp < nz; ++zp) {
                const double2 bb = bpin[zp];
                const double h1 = __ldg(&ops.PpinT[(size_t)zp * nz + z]);
                a.x = fma(h1, bb.x, a.x);
                a.y = fma(h1, bb.y, a.y);
            }
            PHI[(size_t)z * g.nm] = a;
        }
        return;
    }
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int c = t / he, k = t - c * he;
        const int m = m0 + c;
        if (m >= g.nm || (sp.rhs_only && m != 0)) continue;
        Pair x;
        if (m == 0) {
            double2 a = make_double2(0.0, 0.0), b = a;
            for (int zp = 0; zp < nz; ++zp) {
                const double2 bb = bpin[zp];
                const double h1 = __ldg(&ops.PpinT[(size_t)zp * nz + k]);
                const double h2 = __ldg(&ops.PpinT[(size_t)zp * nz + nz - 1 - k]);
                a.x = fma(h1, bb.x, a.x); a.y = fma(h1, bb.y, a.y);
                b.x = fma(h2, bb.x, b.x); b.y = fma(h2, bb.y, b.y);
            }
            x.a = a;
            x.b = b;
        } else {
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            x = inv_apply(ops.PinvF + (size_t)mode_q(ky, kx, g.ny, g.nxhp) * qstride, tb, k, c, tc, he, ho);
        }
        PHI[(size_t)k * g.nm + m] = x.a;
        if (k < ho) PHI[(size_t)(nz - 1 - k) * g.nm + m] = x.b;
    }
}

// The per-mode Poisson inverses applied on the integer pipes.  The folded
// rows are stored in 58-bit fixed point (Ops::PinvI: round(G[k][j]
// 2^(58 - e_k)), row exponents e_k), each mode column of the right-hand side
// in 53-bit fixed point before its even/odd fold (B = round(b 2^(54 - f_c)),
// one power of two 2^(f_c - 1) >= its largest |re|, |im|, so the exact integer
// fold stays within 2^54), and each row's products are summed exactly and
// rounded once: x_k = S 2^(e_k + f_c - 112), with the operands' roundings
// (2^-55 of the column scale, 2^-59 of the row scale per term) and one final
// rounding of 2^-57 of their product: an FP64 dot product's bound.  The exact products are 32-bit multiply-adds
// into 64-bit partial sums: A = a1 2^29 + a0, B = b1 2^27 + b0 (a0 in
// [0, 2^29), b0 in [0, 2^27)), four limb products below 2^56 each, so the
// partial sums of up to 65 terms stay below 2^63 and are combined in 128 bits
// once per output.  GB300's integer multiply-add rate is several times its
// FP64 FMA rate.
struct FxAcc {
    long long p00, p01, p10, p11;  // weights 2^0, 2^27, 2^29, 2^56
};

__device__ __forceinline__ void fx_mad(long long& acc, int a, int b) {  // acc += a b, one 32 x 32 + 64 multiply-add
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(a), "r"(b));
}

__device__ __forceinline__ void fx_mac(FxAcc& acc, int a0, int a1, int b0, int b1) {
    fx_mad(acc.p00, a0, b0);
    fx_mad(acc.p01, a0, b1);
    fx_mad(acc.p10, a1, b0);
    fx_mad(acc.p11, a1, b1);
}

__device__ __forceinline__ double fx_row_value(const FxAcc& acc, int e2) {
    const unsigned __int128 u = (unsigned __int128)(__int128)acc.p00 + ((unsigned __int128)(__int128)acc.p01 << 27) +
                                ((unsigned __int128)(__int128)acc.p10 << 29) +
                                ((unsigned __int128)(__int128)acc.p11 << 56) + ((unsigned __int128)1 << 55);
    const long long T = (long long)((__int128)u >> 56);  // |S| < 2^119: |T| < 2^63
    return i2d_scaled(T, e2 + 56);
}

// A folded column value (|U| <= 2^54) as the limbs (b0, b1) of its re and im
// parts: int4 {re b0, re b1, im b0, im b1}.
__device__ __forceinline__ int4 fx_limbs(long long re, long long im) {
    return make_int4((int)(re & 0x7FFFFFF), (int)(re >> 27), (int)(im & 0x7FFFFFF), (int)(im >> 27));
}

// Modes per CTA of the solve: their fixed-point inverses are staged in shared
// memory (at most 64 KB of them, at least one mode), and one thread takes one
// folded row of one mode (at most 512 rows).
__host__ __device__ inline int fx_solve_modes(int nz) {
    const int ho = nz / 2, he = nz - ho;
    int t = (int)(65536 / (fx_qstride(he, ho) * sizeof(long long)));
    if (t * nz > 512) t = 512 / nz;
    return t < 1 ? 1 : t;
}
__host__ __device__ inline int fx_solve_threads(int nz) { return (nz * fx_solve_modes(nz) + 31) / 32 * 32; }
__host__ __device__ inline size_t fx_solve_smem(int nz) {
    const int ho = nz / 2, he = nz - ho, tc = fx_solve_modes(nz);
    return (size_t)tc * fx_qstride(he, ho) * sizeof(long long) + (2 * (size_t)nz * tc + nz) * sizeof(double2) +
           (size_t)tc * sizeof(int);
}

// The Poisson solve of pressure_body for a right-hand side already in PHI
// (unfolded, as pressure_body forms it), fx_solve_modes(nz) modes from
// bx tc: the modes' fixed-point inverses are copied into shared memory with
// cp.async (16-byte pieces, all in flight at once) while the CTA stages the
// unfolded columns, takes each column's power of two and folds it in fixed
// point; then each thread applies one folded row (above; the pinned mode
// (0,0) unfolded, with its FP64 inverse), and the results are unfolded over
// the right-hand side.  A CTA reads its tile whole before it writes, so the
// solve is in place.  A column with a non-finite entry gets NaN throughout.
__device__ __forceinline__ void pressure_solve_body(const GridDev& g, const Ops& ops, double2* __restrict__ PHI,
                                                    int bx) {
    extern __shared__ __align__(16) unsigned char smc[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    const int tc = fx_solve_modes(nz), tsz = nz * tc;
    const size_t qs = fx_qstride(he, ho);
    long long* sG = reinterpret_cast<long long*>(smc);                  // inverses of the tile's modes [tc][qs]
    double2* su = reinterpret_cast<double2*>(sG + (size_t)tc * qs);   // unfolded columns [nz][tc], then results
    int4* tb = reinterpret_cast<int4*>(su + tsz);                      // folded columns in fixed point (limbs)
    double2* bpin = su + 2 * tsz;                                      // unfolded rhs of mode (0,0)
    int* sF = reinterpret_cast<int*>(bpin + nz);                       // column exponents
    const int m0 = bx * tc;
    {
        const int n16 = (int)(qs / 2);  // 16-byte pieces per mode
        for (int c = 0; c < tc; ++c) {
            const int m = m0 + c;
            if (m >= g.nm || m == 0) continue;
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            const long long* src = ops.PinvI + (size_t)mode_q(ky, kx, g.ny, g.nxhp) * qs;
            long long* dst = sG + (size_t)c * qs;
            for (int i = threadIdx.x; i < n16; i += blockDim.x) cp_async16(dst + 2 * i, src + 2 * i);
        }
        cp_async_commit();
    }
    for (int t = threadIdx.x; t < tsz; t += blockDim.x) {
        const int z = t / tc, c = t - z * tc;
        const int m = m0 + c;
        const double2 v = m < g.nm ? PHI[(size_t)z * g.nm + m] : make_double2(0.0, 0.0);
        su[t] = v;
        if (m == 0) bpin[z] = v;
    }
    __syncthreads();
    {  // one warp per column: the power of two of its largest |re|, |im|
        const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        for (int c = w; c < tc; c += blockDim.x >> 5) {
            unsigned long long mx = 0;
            for (int z = l; z < nz; z += 32) {
                const double2 v = su[z * tc + c];
                const unsigned long long ax = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFULL;
                const unsigned long long ay = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFULL;
                mx = ax > mx ? ax : mx;
                mx = ay > mx ? ay : mx;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
                mx = v > mx ? v : mx;
            }
            if (l == 0) sF[c] = mx >= 0x7FF0000000000000ULL ? INT_MIN : tc_exponent(mx) + 1;
        }
    }
    __syncthreads();
    // fold in fixed point: even rows k < he (pair sums), odd rows he + k (differences)
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int f = sF[c];
        if (f == INT_MIN) continue;  // not read
        const double2 a = su[k * tc + c];
        const long long ax = tc_fixed(a.x, f), ay = tc_fixed(a.y, f);
        if (k < ho) {
            const double2 b = su[(nz - 1 - k) * tc + c];
            const long long bx2 = tc_fixed(b.x, f), by = tc_fixed(b.y, f);
            tb[k * tc + c] = fx_limbs(ax + bx2, ay + by);
            tb[(he + k) * tc + c] = fx_limbs(ax - bx2, ay - by);
        } else {
            tb[k * tc + c] = fx_limbs(ax, ay);
        }
    }
    cp_async_wait_all();
    __syncthreads();  // the folded tile and every thread's operator pieces
    // one folded row r of one column per thread (rows of a column on adjacent lanes)
    for (int t = threadIdx.x; t < tsz; t += blockDim.x) {
        const int c = t / nz, r = t - c * nz;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        if (m == 0) {  // the pinned mode: output level r, unfolded, FP64
            double2 a = make_double2(0.0, 0.0);
            for (int zp = 0; zp < nz; ++zp) {
                const double2 bb = bpin[zp];
                const double h1 = __ldg(&ops.PpinT[(size_t)zp * nz + r]);
                a.x = fma(h1, bb.x, a.x);
                a.y = fma(h1, bb.y, a.y);
            }
            PHI[(size_t)r * g.nm] = a;
            continue;
        }
        const int f = sF[c];
        double2 x;
        if (f == INT_MIN) {
            x.x = x.y = __longlong_as_double(0x7FF8000000000000LL);
        } else {
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            const size_t q = (size_t)mode_q(ky, kx, g.ny, g.nxhp);
            const bool even = r < he;
            const int n = even ? he : ho, k = even ? r : r - he;
            const long long* G = sG + (size_t)c * qs + (even ? 0 : (size_t)he * he) + k;
            const int4* bcol = tb + (even ? 0 : he * tc) + c;
            FxAcc sx{}, sy{};
#pragma unroll 4
            for (int j = 0; j < n; ++j, G += n, bcol += tc) {
                const long long a = *G;
                const int a0 = (int)(a & 0x1FFFFFFF), a1 = (int)(a >> 29);
                const int4 b = *bcol;
                fx_mac(sx, a0, a1, b.x, b.y);
                fx_mac(sy, a0, a1, b.z, b.w);
            }
            const int e2 = __ldg(&ops.PinvE[q * nz + r]) + f - 112;
            x = make_double2(fx_row_value(sx, e2), fx_row_value(sy, e2));
        }
        su[r * tc + c] = x;  // su's column c was last read by the fold, before the barrier
    }
    __syncthreads();
    // unfold: phi_k = pe_k + po_k, phi_nz-1-k = pe_k - po_k
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm || m == 0) continue;
        const double2 pe = su[k * tc + c];
        if (k < ho) {
            const double2 po = su[(he + k) * tc + c];
            PHI[(size_t)k * g.nm + m] = make_double2(pe.x + po.x, pe.y + po.y);
            PHI[(size_t)(nz - 1 - k) * g.nm + m] = make_double2(pe.x - po.x, pe.y - po.y);
        } else {
            PHI[(size_t)k * g.nm + m] = pe;
        }
    }
}

__global__ void __launch_bounds__(512) k_pressure_solve(GridDev g, Ops ops, double2* __restrict__ PHI) {
    pressure_solve_body(g, ops, PHI, blockIdx.x);
}

// The divergence right-hand side of pressure_body (strong form) from D1.w*,
// written unfolded into PHI for pressure_solve_body
struct PresRhsTcOp {
    static constexpr int kFields = 1;
    StepParams sp;
    const double2* __restrict__ US;
    const double2* __restrict__ VS;
    const double2* __restrict__ WS;
    double2* __restrict__ PHI;
    __device__ const double2* field(int) const { return WS; }
    // the right-hand side at level z of mode m from d = D1.w* there
    __device__ void out_level(const GridDev& g, const Ops& ops, int m, int z, const double2* d) const {
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        PHI[(size_t)z * g.nm + m] = pressure_rhs(g, ops, sp, z, m, mi, US, VS, d[0]);
    }
};

__global__ void __launch_bounds__(256) k_pressure(GridDev g, Ops ops, StepParams sp,
                                                  const double2* __restrict__ US,
                                                  const double2* __restrict__ VS,
                                                  const double2* __restrict__ WS,
                                                  double2* __restrict__ PHI, int tc) {
    pressure_body(g, ops, sp, US, VS, WS, PHI, tc, blockIdx.x);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------ jacgs
// jacgs (DNS_pressure_BC_2D.f90:2361-2476) for one real system per warp:
// (a S[off+i][off+j] + diag(dg)) x = b, n <= 160 unknowns, rows i = lane +
// 32 s held in registers, the search direction shared through the warp's
// shared-memory vector for the product with S (S staged in shared memory).
// Jacobi preconditioner, x0 = 0, small = 1e-30 guards, at most 500
// iterations, stop when |r|_2 <= tol |r0|_2 (every lane takes the same
// decision: the reductions are butterflies).  A system that does not
// converge keeps its last iterate, as the reference uses its partial result.
constexpr int kPcgWarps = 8;
constexpr int kPcgRows = 5;  // ceil(160 / 32)

__device__ void warp_pcg(const double* __restrict__ S, int lds, int off, int n, double a, const double* dg,
                         const double* bl, double* xl, double* pw, double tol) {
    const int lane = threadIdx.x & 31;
    const double small = 1.0e-30;
    double r[kPcgRows], q[kPcgRows], p[kPcgRows], dinv[kPcgRows], ap[kPcgRows];
    double rr = 0.0;
#pragma unroll
    for (int s = 0; s < kPcgRows; ++s) {
        const int i = lane + 32 * s;
        xl[s] = 0.0;
        r[s] = q[s] = p[s] = dinv[s] = ap[s] = 0.0;
        if (i < n) {
            const double d = a * S[(size_t)(off + i) * lds + off + i] + dg[s];
            dinv[s] = fabs(d) > small ? 1.0 / d : 1.0;
            r[s] = bl[s];
            q[s] = r[s] * dinv[s];
            p[s] = q[s];
            rr = fma(r[s], r[s], rr);
        }
    }
    const double res0 = sqrt(warp_sum(rr));
    if (!(res0 > 0.0)) return;
    for (int it = 0; it < 500; ++it) {
#pragma unroll
        for (int s = 0; s < kPcgRows; ++s)
            if (lane + 32 * s < n) pw[lane + 32 * s] = p[s];
        __syncwarp();
        double qr = 0.0, pa = 0.0;
#pragma unroll
        for (int s = 0; s < kPcgRows; ++s) {
            const int i = lane + 32 * s;
            if (i < n) {
                const double* row = S + (size_t)(off + i) * lds + off;
                double acc = 0.0;
                for (int j = 0; j < n; ++j) acc = fma(row[j], pw[j], acc);
                ap[s] = fma(a, acc, dg[s] * p[s]);
                qr = fma(q[s], r[s], qr);
                pa = fma(p[s], ap[s], pa);
            }
        }
        __syncwarp();
        const double qdr = warp_sum(qr);
        const double alfa = qdr / (warp_sum(pa) + small);
        double qn = 0.0, rn = 0.0;
#pragma unroll
        for (int s = 0; s < kPcgRows; ++s) {
            if (lane + 32 * s < n) {
                xl[s] = fma(alfa, p[s], xl[s]);
                r[s] = fma(-alfa, ap[s], r[s]);
                q[s] = r[s] * dinv[s];
                qn = fma(q[s], r[s], qn);
                rn = fma(r[s], r[s], rn);
            }
        }
        const double beta = warp_sum(qn) / (qdr + small);
#pragma unroll
        for (int s = 0; s < kPcgRows; ++s)
            if (lane + 32 * s < n) p[s] = fma(beta, p[s], q[s]);
        if (sqrt(warp_sum(rn)) <= tol * res0) break;
    }
}

// Poisson, every mode but (0,0): (S + k^2 w ybar/2) phi = -b, b in PHI.
__global__ void __launch_bounds__(32 * kPcgWarps) k_pcg_poisson(GridDev g, Ops ops, double2* PHI, double tol) {
    extern __shared__ double psm[];
    const int nz = g.nz;
    for (int t = threadIdx.x; t < nz * nz; t += blockDim.x) psm[t] = ops.S[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* pw = psm + nz * nz + warp * nz;
    const long long sid = (long long)blockIdx.x * kPcgWarps + warp;
    if (sid >= 2LL * (g.nm - 1)) return;
    const int m = 1 + (int)(sid >> 1), part = (int)(sid & 1);
    const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
    const double k2 = __ldg(&ops.ksq[mode_q(ky, kx, g.ny, g.nxhp)]);
    double* ph = reinterpret_cast<double*>(PHI);
    double dg[kPcgRows], bl[kPcgRows], xl[kPcgRows];
#pragma unroll
    for (int s = 0; s < kPcgRows; ++s) {
        const int i = lane + 32 * s;
        dg[s] = bl[s] = 0.0;
        if (i < nz) {
            dg[s] = k2 * __ldg(&ops.wh[i]);
            bl[s] = -ph[2 * ((size_t)i * g.nm + m) + part];
        }
    }
    warp_pcg(psm, nz, 0, nz, 1.0, dg, bl, xl, pw, tol);
#pragma unroll
    for (int s = 0; s < kPcgRows; ++s) {
        const int i = lane + 32 * s;
        if (i < nz) ph[2 * ((size_t)i * g.nm + m) + part] = xl[s];
    }
}

// Helmholtz, every mode, component and part: the interior system
// (f S_II + diag((1 + f k^2) w ybar/2)) x_I = b_I - (f S_I1 x_1 + f S_In x_n),
// b and the wall values x_1, x_n as the viscous kernel left them in Out.
__global__ void __launch_bounds__(32 * kPcgWarps) k_pcg_helmholtz(GridDev g, Ops ops, StepParams sp, Fields Out,
                                                                   double tol) {
    extern __shared__ double psm[];
    const int nz = g.nz;
    for (int t = threadIdx.x; t < nz * nz; t += blockDim.x) psm[t] = ops.S[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* pw = psm + nz * nz + warp * nz;
    const long long sid = (long long)blockIdx.x * kPcgWarps + warp;
    if (sid >= 6LL * g.nm) return;
    const int m = (int)(sid / 6), rem = (int)(sid % 6), comp = rem >> 1, part = rem & 1;
    const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
    const double k2 = __ldg(&ops.ksq[mode_q(ky, kx, g.ny, g.nxhp)]);
    const double f = sp.helm_f;
    double* o = reinterpret_cast<double*>(fptr(Out, comp));
    const double bc1 = o[2 * (size_t)m + part];
    const double bc2 = o[2 * ((size_t)(nz - 1) * g.nm + m) + part];
    double dg[kPcgRows], bl[kPcgRows], xl[kPcgRows];
    const int n = nz - 2;
#pragma unroll
    for (int s = 0; s < kPcgRows; ++s) {
        const int i = lane + 32 * s, z = i + 1;
        dg[s] = bl[s] = 0.0;
        if (i < n) {
            dg[s] = (1.0 + f * k2) * __ldg(&ops.wh[z]);
            bl[s] = o[2 * ((size_t)z * g.nm + m) + part] - (__ldg(&ops.S0[z]) * bc1 + __ldg(&ops.Sn[z]) * bc2);
        }
    }
    warp_pcg(psm, nz, 1, n, f, dg, bl, xl, pw, tol);
#pragma unroll
    for (int s = 0; s < kPcgRows; ++s) {
        const int i = lane + 32 * s;
        if (i < n) o[2 * ((size_t)(i + 1) * g.nm + m) + part] = xl[s];
    }
}

// dynamic shared memory of the jacgs kernels: S and one vector per warp
size_t pcg_smem(const GridDev& g) { return ((size_t)g.nz * g.nz + (size_t)kPcgWarps * g.nz) * sizeof(double); }

// ------------------------------------------------------------------ jst4 stages
// stage state of runge_kutta_convection (DNS_pressure_BC_2D.f90:985-993)
// lifted to 3D: out = F + coef * mask(S), wall levels zeroed (apply_wall_bc).
template <typename SrcC>
__global__ void k_rk_stage(GridDev g, StepParams sp, double coef, Fields F, FieldsT<SrcC> Src, Fields Out) {
    const size_t per = (size_t)g.nz * g.nm, total = 3 * per;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int comp = (int)(t / per);
        const size_t o = t - comp * per;
        const int z = (int)(o / g.nm), m = (int)(o - (size_t)z * g.nm);
        double2 r = make_double2(0.0, 0.0);
        if (z != 0 && z != g.nz - 1) {
            double2 sv = to_d2(fptr(Src, comp)[o]);
            if (sp.dealias) {
                const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
                const int kyi = ky <= g.ny / 2 ? ky : g.ny - ky;
                if (kx > sp.kx_max || kyi > sp.ky_max) sv = make_double2(0.0, 0.0);
            }
            const double2 fv = fptr(F, comp)[o];
            r = make_double2(fv.x + coef * sv.x, fv.y + coef * sv.y);
        }
        fptr(Out, comp)[o] = r;
    }
}

// ------------------------------------------------------------------ correction
// pressure_correction_3d (3D:1903-1929): u = u* - dt grad(phi), p += phi,
// grad_p_prev = grad(p_total); only its wall planes are consumed (3D:1325-1326).
__device__ __forceinline__ void correction_body(GridDev g, Ops ops, StepParams sp,
                                                const double2* __restrict__ US,
                                                const double2* __restrict__ VS,
                                                const double2* __restrict__ WS,
                                                const double2* __restrict__ PHI,
                                                double2* __restrict__ U, double2* __restrict__ V,
                                                double2* __restrict__ W, double2* __restrict__ P,
                                                double2* __restrict__ GP, int tc, int bx) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    double2* tp = sm;
    const int m0 = bx * tc;
    fold_load(tp, PHI, g, m0, tc, he, ho);
    __syncthreads();
    const double dt = sp.dt;
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        const Pair dz = anti_apply(ops.D1e, ops.D1o, tp, k, c, tc, he, ho);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const int npt = (k < ho) ? 2 : 1;
        for (int p = 0; p < npt; ++p) {
            const int z = p ? nz - 1 - k : k;
            const double2 d = p ? dz.b : dz.a;
            const size_t o = (size_t)z * g.nm + m;
            const double2 ph = PHI[o];
            const double2 px = i_times(mi.ax, ph), py = i_times(mi.ay, ph);
            const double2 us = US[o], vs = VS[o], ws = WS[o];
            store_projection(sp, z, g.nz, o, make_double2(us.x - dt * px.x, us.y - dt * px.y),
                             make_double2(vs.x - dt * py.x, vs.y - dt * py.y),
                             make_double2(ws.x - dt * d.x, ws.y - dt * d.y), U, V, W);
            double2 pp = P[o];
            pp.x += ph.x;
            pp.y += ph.y;
            P[o] = pp;
            if (z == 0 || z == nz - 1) {
                const int wall = (z == 0) ? 0 : 1;
                GP[(size_t)wall * g.nm + m] = i_times(mi.ax, pp);
                GP[(size_t)(2 + wall) * g.nm + m] = i_times(mi.ay, pp);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_correction(GridDev g, Ops ops, StepParams sp,
                                                    const double2* __restrict__ US,
                                                    const double2* __restrict__ VS,
                                                    const double2* __restrict__ WS,
                                                    const double2* __restrict__ PHI,
                                                    double2* __restrict__ U, double2* __restrict__ V,
                                                    double2* __restrict__ W, double2* __restrict__ P,
                                                    double2* __restrict__ GP, int tc) {
    correction_body(g, ops, sp, US, VS, WS, PHI, U, V, W, P, GP, tc, blockIdx.x);
}

// Wall-plane gradients of p_total alone (used when the state is set).
__global__ void k_grad_walls(GridDev g, Ops ops, const double2* __restrict__ P, double2* __restrict__ GP) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= g.nm) return;
    const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
    for (int wall = 0; wall < 2; ++wall) {
        const double2 p = P[(size_t)(wall ? g.nz - 1 : 0) * g.nm + m];
        GP[(size_t)wall * g.nm + m] = i_times(mi.ax, p);
        GP[(size_t)(2 + wall) * g.nm + m] = i_times(mi.ay, p);
    }
}

// apply_boundary_conditions_3d (3D:1953-1972): wall planes := 0 (the wall
// arrays are all zero, 3D:987-999), i.e. spectral planes k=1, nz := 0.
__device__ __forceinline__ void apply_bc_body(GridDev g, double2* U, double2* V, double2* W, int bx) {
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= 2 * g.nm) return;
    const int wall = i / g.nm, m = i - wall * g.nm;
    const size_t o = (size_t)(wall ? g.nz - 1 : 0) * g.nm + m;
    const double2 z = make_double2(0.0, 0.0);
    U[o] = z;
    V[o] = z;
    W[o] = z;
}

__global__ void k_apply_bc(GridDev g, double2* U, double2* V, double2* W) {
    apply_bc_body(g, U, V, W, blockIdx.x);
}

// Divergence spectrum DX u + DY v + Dz w (compute_divergence_3d, 3D:1858-1879).
__global__ void __launch_bounds__(256) k_divergence(GridDev g, Ops ops, const double2* __restrict__ U,
                                                    const double2* __restrict__ V,
                                                    const double2* __restrict__ W,
                                                    double2* __restrict__ DIV, int tc) {
    extern __shared__ double2 sm[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    double2* tw = sm;
    const int m0 = blockIdx.x * tc;
    fold_load(tw, W, g, m0, tc, he, ho);
    __syncthreads();
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        const Pair dz = anti_apply(ops.D1e, ops.D1o, tw, k, c, tc, he, ho);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const int npt = (k < ho) ? 2 : 1;
        for (int p = 0; p < npt; ++p) {
            const int z = p ? nz - 1 - k : k;
            const double2 d = p ? dz.b : dz.a;
            const size_t o = (size_t)z * g.nm + m;
            const double2 hx = i_times(mi.ax, U[o]);
            const double2 hy = i_times(mi.ay, V[o]);
            DIV[o] = make_double2((hx.x + hy.x) + d.x, (hx.y + hy.y) + d.y);
        }
    }
}

// ------------------------------------------------------------------ mixed precision
// FP32 vorticity: the FP64 spectra of u, v, w are rounded to FP32 once and
// omega is formed in FP32 (folded FP32 D); outputs u, v, w, ox, oy, oz (FP32)
// feed the FP32 inverse transforms of the nonlinear term.
__device__ __forceinline__ void fold_load32(float2* tile, const double2* __restrict__ src, const GridDev& g,
                                            int m0, int tc, int he, int ho) {
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        float2 fe = make_float2(0.f, 0.f), fo = fe;
        if (m < g.nm) {
            const double2 a = src[(size_t)k * g.nm + m];
            if (k < ho) {
                const double2 b = src[(size_t)(g.nz - 1 - k) * g.nm + m];
                const float ax = (float)a.x, ay = (float)a.y, bx = (float)b.x, by = (float)b.y;
                fe = make_float2(ax + bx, ay + by);
                fo = make_float2(ax - bx, ay - by);
            } else {
                fe = make_float2((float)a.x, (float)a.y);
            }
        }
        tile[t] = fe;
        if (k < ho) tile[(he + k) * tc + c] = fo;
    }
}

// sum_j erow[j] a[j] and sum_j erow[j] b[j] over j < len for two folded
// tile parts a, b (column stride tc), each row entry loaded once for both
__device__ __forceinline__ void fold_dot32x2(const float* __restrict__ erow, const float2* a, const float2* b,
                                             int len, int tc, int c, float2& ra, float2& rb) {
    float2 sa = make_float2(0.f, 0.f), sb = sa;
#pragma unroll 4
    for (int j = 0; j < len; ++j) {
        const float e = __ldg(&erow[j]);
        const float2 x = a[j * tc + c], y = b[j * tc + c];
        sa.x = fmaf(e, x.x, sa.x);
        sa.y = fmaf(e, x.y, sa.y);
        sb.x = fmaf(e, y.x, sb.x);
        sb.y = fmaf(e, y.y, sb.y);
    }
    ra = sa;
    rb = sb;
}

__device__ __forceinline__ void vorticity_mixed_body(GridDev g, MixedOps mx, Ops ops,
                                                     const double2* __restrict__ U,
                                                     const double2* __restrict__ V,
                                                     const double2* __restrict__ W, FFields out, int tc, int bx) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* tu = reinterpret_cast<float2*>(smraw);
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    float2* tv = tu + nz * tc;
    const int m0 = bx * tc;
    fold_load32(tu, U, g, m0, tc, he, ho);
    fold_load32(tv, V, g, m0, tc, he, ho);
    __syncthreads();
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        if (m >= g.nm) continue;
        float2 due, dve, duo = make_float2(0.f, 0.f), dvo = duo;
        fold_dot32x2(mx.D1e + (size_t)k * ho, tu + he * tc, tv + he * tc, ho, tc, c, due, dve);
        if (k < ho) fold_dot32x2(mx.D1o + (size_t)k * he, tu, tv, he, tc, c, duo, dvo);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const float ax = (float)mi.ax, ay = (float)mi.ay;
        const int npt = (k < ho) ? 2 : 1;
        for (int p = 0; p < npt; ++p) {
            const int z = p ? nz - 1 - k : k;
            const size_t o = (size_t)z * g.nm + m;
            const double2 wd = W[o], ud = U[o], vd = V[o];
            const float2 w = make_float2((float)wd.x, (float)wd.y);
            const float2 u = make_float2((float)ud.x, (float)ud.y);
            const float2 v = make_float2((float)vd.x, (float)vd.y);
            const float2 du = p ? make_float2(due.x - duo.x, due.y - duo.y) : make_float2(due.x + duo.x, due.y + duo.y);
            const float2 dv = p ? make_float2(dve.x - dvo.x, dve.y - dvo.y) : make_float2(dve.x + dvo.x, dve.y + dvo.y);
            // (i a) f = (-a f.y, a f.x)
            out.p[0][o] = u;
            out.p[1][o] = v;
            out.p[2][o] = w;
            out.p[3][o] = make_float2(-ay * w.y - dv.x, ay * w.x - dv.y);          // wy - vz
            out.p[4][o] = make_float2(du.x + ax * w.y, du.y - ax * w.x);           // uz - wx
            out.p[5][o] = make_float2(-ax * v.y + ay * u.y, ax * v.x - ay * u.x);  // vx - uy
        }
    }
}

__global__ void __launch_bounds__(256) k_vorticity_mixed(GridDev g, MixedOps mx, Ops ops,
                                                         const double2* __restrict__ U,
                                                         const double2* __restrict__ V,
                                                         const double2* __restrict__ W, FFields out, int tc) {
    vorticity_mixed_body(g, mx, ops, U, V, W, out, tc, blockIdx.x);
}

__device__ __forceinline__ void products32_body(FRFields in, FRFields out, size_t n, int bx, int gx) {
    const size_t stride = (size_t)gx * blockDim.x;
    for (size_t i = (size_t)bx * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float u = in.p[0][i], v = in.p[1][i], w = in.p[2][i];
        const float ox = in.p[3][i], oy = in.p[4][i], oz = in.p[5][i];
        out.p[0][i] = v * oz - w * oy;
        out.p[1][i] = w * ox - u * oz;
        out.p[2][i] = u * oy - v * ox;
    }
}

__global__ void k_products32(FRFields in, FRFields out, size_t n) {
    products32_body(in, out, n, blockIdx.x, gridDim.x);
}

// (The viscous and pressure kernels below convert between FP64 and FP32 with
// cvt.cuh's integer-pipe d2f / f2d: measured 55 -> 51 us and 76 -> 71 us at
// 128x128x65.  The vorticity above keeps the hardware conversions, which
// measured faster there.)
//
// Viscous step as an increment in the eigenbasis of the interior Helmholtz
// problem.  With S_II V = M_II V Lambda, V^T M_II V = I, and the identity
// M_I (d2 u)_I = -(S u)_I (LGL quadrature is exact for these products), the
// reference's system H_II x_I = M_I rhs_I - 2 f (S_I1 bc1 + S_In bc2) gives
//   x_I - u_I = V y,  y_j = -(c+f)(k^2+l_j) g_j ut_j
//                          + g_j (dt St_j - c (s0_j u_1 + sn_j u_n) - 2f (s0_j bc1 + sn_j bc2))
// with g_j = 1/(1 + f(k^2 + l_j)), ut = V^T M_I u_I, St = V^T M_I S_I,
// s0 = V^T S_I1, sn = V^T S_In (c = explicit-diffusion factor, f = theta dt/Re).
// All products are FP32; the increment is added to the FP64 state, so the
// FP32 error scales with the (small) increment.  Mode (0,0) is skipped: it is
// advanced in FP64 by k_viscous.
__device__ __forceinline__ void viscous_mixed_body(GridDev g, MixedOps mx, Ops ops, StepParams sp,
                                                   Fields F, FFields Src, const double2* __restrict__ GP,
                                                   Fields Out, int tc, int bx, bool stage_mats = true) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int hei = mx.hei, hoi = mx.hoi, pe4 = mx.pe4, po4 = mx.po4;
    const int nr = pe4 + po4;        // folded rows (even block, then odd block)
    const int tsz = nr * tc;
    float4* sAe = reinterpret_cast<float4*>(smraw);    // AeT [hei][pe4/4]
    float4* sAo = sAe + (size_t)hei * (pe4 / 4);        // AoT [hoi][po4/4]
    float4* sBe = sAo + (size_t)hoi * (po4 / 4);        // BeT [hei][pe4/4]
    float4* sBo = sBe + (size_t)hei * (pe4 / 4);        // BoT [hoi][po4/4]
    float2* tu = reinterpret_cast<float2*>(sBo + (size_t)hoi * (po4 / 4));  // [nr][tc] folded interior u
    float2* ts = tu + tsz;                              // [nr][tc] folded interior S
    float2* ty = ts + tsz;                              // [nr][tc] eigen-space update
    float4* tw = reinterpret_cast<float4*>(ty + tsz);   // [tc] wall terms
    float* tk = reinterpret_cast<float*>(tw + tc);      // [tc] k^2 (-1: skip; <= -2: masked source)
    const int m0 = bx * tc;
    if (stage_mats) {  // the eigenbasis matrices (a persistent CTA stages them once)
        const float4* A = reinterpret_cast<const float4*>(mx.AeT);
        for (int t = threadIdx.x; t < hei * (pe4 / 4); t += blockDim.x) sAe[t] = __ldg(&A[t]);
        A = reinterpret_cast<const float4*>(mx.AoT);
        for (int t = threadIdx.x; t < hoi * (po4 / 4); t += blockDim.x) sAo[t] = __ldg(&A[t]);
        A = reinterpret_cast<const float4*>(mx.BeT);
        for (int t = threadIdx.x; t < hei * (pe4 / 4); t += blockDim.x) sBe[t] = __ldg(&A[t]);
        A = reinterpret_cast<const float4*>(mx.BoT);
        for (int t = threadIdx.x; t < hoi * (po4 / 4); t += blockDim.x) sBo[t] = __ldg(&A[t]);
    }
    const float dt = d2f(sp.dt), cf = d2f(sp.cn_fac), ff = d2f(sp.helm_f);
    for (int comp = 0; comp < 3; ++comp) {
        // fold the interior column: even rows k < hei, odd rows pe4 + k
        for (int t = threadIdx.x; t < pe4 * tc; t += blockDim.x) {
            const int k = t / tc, c = t - k * tc;
            const int m = m0 + c;
            float2 se = make_float2(0.f, 0.f), de = se, ss = se, ds = se;
            if (m < g.nm && k < hei) {
                const size_t o1 = (size_t)(1 + k) * g.nm + m;
                const double2 a = fptr(F, comp)[o1];
                const float2 sa = fptr(Src, comp)[o1];
                const float ax = d2f(a.x), ay = d2f(a.y);
                if (k < hoi) {
                    const size_t o2 = (size_t)(g.nz - 2 - k) * g.nm + m;
                    const double2 b = fptr(F, comp)[o2];
                    const float2 sb = fptr(Src, comp)[o2];
                    const float bx = d2f(b.x), by = d2f(b.y);
                    se = make_float2(ax + bx, ay + by);
                    de = make_float2(ax - bx, ay - by);
                    ss = make_float2(sa.x + sb.x, sa.y + sb.y);
                    ds = make_float2(sa.x - sb.x, sa.y - sb.y);
                } else {
                    se = make_float2(ax, ay);
                    ss = sa;
                }
            }
            tu[t] = se;
            ts[t] = ss;
            if (k < po4) {
                tu[(pe4 + k) * tc + c] = de;
                ts[(pe4 + k) * tc + c] = ds;
            }
        }
        for (int c = threadIdx.x; c < tc; c += blockDim.x) {
            const int m = m0 + c;
            float k2 = -1.f;
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (m < g.nm && m != 0) {
                const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
                bool keep = true;
                if (sp.dealias) {
                    const int kyi = ky <= g.ny / 2 ? ky : g.ny - ky;
                    keep = !(kx > sp.kx_max || kyi > sp.ky_max);
                }
                k2 = d2f(__ldg(&ops.ksq[mode_q(ky, kx, g.ny, g.nxhp)]));
                if (!keep) k2 = -2.f - k2;  // masked source: flagged by the sign
                const double2 u0 = fptr(F, comp)[(size_t)m], un = fptr(F, comp)[(size_t)(g.nz - 1) * g.nm + m];
                double2 b1 = make_double2(0.0, 0.0), b2 = b1;
                if (comp < 2) {
                    const double2 g1 = GP[(size_t)(2 * comp) * g.nm + m];
                    const double2 g2 = GP[(size_t)(2 * comp + 1) * g.nm + m];
                    b1 = make_double2(-sp.dt * g1.x, -sp.dt * g1.y);
                    b2 = make_double2(-sp.dt * g2.x, -sp.dt * g2.y);
                }
                w = make_float4(cf * d2f(u0.x) + 2.0f * ff * d2f(b1.x), cf * d2f(u0.y) + 2.0f * ff * d2f(b1.y),
                                cf * d2f(un.x) + 2.0f * ff * d2f(b2.x), cf * d2f(un.y) + 2.0f * ff * d2f(b2.y));
            }
            tk[c] = k2;
            tw[c] = w;
        }
        __syncthreads();
        // ut, st for 4 eigen-rows of one block (even or odd)
        for (int t = threadIdx.x; t < (nr / 4) * tc; t += blockDim.x) {
            const int jb = t / tc, c = t - jb * tc;
            const int j0 = 4 * jb;
            float k2 = tk[c];
            if (k2 == -1.f) {
                for (int q = 0; q < 4; ++q) ty[(j0 + q) * tc + c] = make_float2(0.f, 0.f);
                continue;
            }
            const bool keep = k2 >= 0.f;
            if (!keep) k2 = -2.f - k2;
            const bool even = j0 < pe4;
            const float4* A = even ? sAe + jb : sAo + (jb - pe4 / 4);
            const int lda = even ? pe4 / 4 : po4 / 4;
            const int len = even ? hei : hoi;
            const float2* cu = tu + (even ? 0 : pe4 * tc);
            const float2* cs = ts + (even ? 0 : pe4 * tc);
            float2 ut[4], st[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) { ut[q] = make_float2(0.f, 0.f); st[q] = ut[q]; }
            for (int i = 0; i < len; ++i) {
                const float4 e = A[i * lda];
                const float2 a = cu[i * tc + c];
                const float2 b = cs[i * tc + c];
                ut[0].x = fmaf(e.x, a.x, ut[0].x); ut[0].y = fmaf(e.x, a.y, ut[0].y);
                ut[1].x = fmaf(e.y, a.x, ut[1].x); ut[1].y = fmaf(e.y, a.y, ut[1].y);
                ut[2].x = fmaf(e.z, a.x, ut[2].x); ut[2].y = fmaf(e.z, a.y, ut[2].y);
                ut[3].x = fmaf(e.w, a.x, ut[3].x); ut[3].y = fmaf(e.w, a.y, ut[3].y);
                st[0].x = fmaf(e.x, b.x, st[0].x); st[0].y = fmaf(e.x, b.y, st[0].y);
                st[1].x = fmaf(e.y, b.x, st[1].x); st[1].y = fmaf(e.y, b.y, st[1].y);
                st[2].x = fmaf(e.z, b.x, st[2].x); st[2].y = fmaf(e.z, b.y, st[2].y);
                st[3].x = fmaf(e.w, b.x, st[3].x); st[3].y = fmaf(e.w, b.y, st[3].y);
            }
            if (!keep) {
#pragma unroll
                for (int q = 0; q < 4; ++q) st[q] = make_float2(0.f, 0.f);
            }
            const float4 w = tw[c];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + q;  // padded rows have lam = s0 = sn = 0 and zero inputs
                const float k2l = k2 + __ldg(&mx.lam[j]);
                const float gj = 1.0f / (1.0f + ff * k2l);
                const float cu_ = -(cf + ff) * k2l * gj;
                const float s0 = __ldg(&mx.s0[j]), sn = __ldg(&mx.sn[j]);
                const float lx = dt * st[q].x - (s0 * w.x + sn * w.z);
                const float ly = dt * st[q].y - (s0 * w.y + sn * w.w);
                ty[j * tc + c] = make_float2(cu_ * ut[q].x + gj * lx, cu_ * ut[q].y + gj * ly);
            }
        }
        __syncthreads();
        // back to the interior levels: 4 output pairs per item
        for (int t = threadIdx.x; t < (pe4 / 4) * tc; t += blockDim.x) {
            const int ib = t / tc, c = t - ib * tc;
            const int m = m0 + c;
            if (tk[c] == -1.f) continue;
            const int i0 = 4 * ib;
            float2 pe[4], po[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) { pe[q] = make_float2(0.f, 0.f); po[q] = pe[q]; }
            for (int j = 0; j < hei; ++j) {
                const float4 e = sBe[j * (pe4 / 4) + ib];
                const float2 y = ty[j * tc + c];
                pe[0].x = fmaf(e.x, y.x, pe[0].x); pe[0].y = fmaf(e.x, y.y, pe[0].y);
                pe[1].x = fmaf(e.y, y.x, pe[1].x); pe[1].y = fmaf(e.y, y.y, pe[1].y);
                pe[2].x = fmaf(e.z, y.x, pe[2].x); pe[2].y = fmaf(e.z, y.y, pe[2].y);
                pe[3].x = fmaf(e.w, y.x, pe[3].x); pe[3].y = fmaf(e.w, y.y, pe[3].y);
            }
            if (i0 < po4) {
                for (int j = 0; j < hoi; ++j) {
                    const float4 e = sBo[j * (po4 / 4) + ib];
                    const float2 y = ty[(pe4 + j) * tc + c];
                    po[0].x = fmaf(e.x, y.x, po[0].x); po[0].y = fmaf(e.x, y.y, po[0].y);
                    po[1].x = fmaf(e.y, y.x, po[1].x); po[1].y = fmaf(e.y, y.y, po[1].y);
                    po[2].x = fmaf(e.z, y.x, po[2].x); po[2].y = fmaf(e.z, y.y, po[2].y);
                    po[3].x = fmaf(e.w, y.x, po[3].x); po[3].y = fmaf(e.w, y.y, po[3].y);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int i = i0 + q;
                if (i >= hei) break;
                const size_t o1 = (size_t)(1 + i) * g.nm + m;
                const double2 u1 = fptr(F, comp)[o1];
                if (i < hoi) {
                    const size_t o2 = (size_t)(g.nz - 2 - i) * g.nm + m;
                    const double2 u2 = fptr(F, comp)[o2];
                    fptr(Out, comp)[o1] = make_double2(u1.x + f2d(pe[q].x + po[q].x), u1.y + f2d(pe[q].y + po[q].y));
                    fptr(Out, comp)[o2] = make_double2(u2.x + f2d(pe[q].x - po[q].x), u2.y + f2d(pe[q].y - po[q].y));
                } else {  // middle level (ni odd)
                    fptr(Out, comp)[o1] = make_double2(u1.x + f2d(pe[q].x), u1.y + f2d(pe[q].y));
                }
            }
            if (ib == 0) {  // x_1 = bc1, x_n = bc2 (identity rows)
                for (int wall = 0; wall < 2; ++wall) {
                    double2 bc = make_double2(0.0, 0.0);
                    if (comp < 2) {
                        const double2 gp = GP[(size_t)(2 * comp + wall) * g.nm + m];
                        bc = make_double2(-sp.dt * gp.x, -sp.dt * gp.y);
                    }
                    fptr(Out, comp)[(size_t)(wall ? g.nz - 1 : 0) * g.nm + m] = bc;
                }
            }
        }
        __syncthreads();
    }
}

// Persistent: a CTA stages the matrices once and takes every gridDim.x-th tile.
__global__ void __launch_bounds__(256) k_viscous_mixed(GridDev g, MixedOps mx, Ops ops, StepParams sp,
                                                       Fields F, FFields Src, const double2* __restrict__ GP,
                                                       Fields Out, int tc) {
    const int ntiles = (g.nm + tc - 1) / tc;
    for (int bx = blockIdx.x; bx < ntiles; bx += gridDim.x) {
        viscous_mixed_body(g, mx, ops, sp, F, Src, GP, Out, tc, bx, bx == (int)blockIdx.x);
        __syncthreads();  // the tile buffers are reused by the next tile
    }
}

// ------------------------------------------------------------------ double-float
// Double-float ("df64") arithmetic on the FP32 pipe for the one contraction of
// the mixed path that needs FP64 accuracy.  A value is hi + lo with hi the
// FP32 rounding of x and lo the FP32 rounding of x - hi (~48 significant bits).
// Products use the exact FMA residual fma(a, b, -a*b); sums use Knuth's
// two-sum, so an n-term dot product is accurate to ~n 2^-48 relative to
// sum |a_i b_i|.  On GB300 one such multiply-add is ~11 FP32 instructions,
// about 6x cheaper than a native FP64 FMA.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_split(double x) {
    DF r;
    r.hi = d2f(x);
    r.lo = d2f(x - f2d(r.hi));
    return r;
}
// s += a * b, a and b double-float
// (the _rn intrinsics are never contracted into FMAs, which would break the
// exactness of the two-sum)
__device__ __forceinline__ void df_mac(DF& s, float ahi, float alo, float bhi, float blo) {
    const float p = __fmul_rn(ahi, bhi);
    float e = fmaf(ahi, bhi, -p);
    e = fmaf(ahi, blo, e);
    e = fmaf(alo, bhi, e);
    const float t = __fadd_rn(s.hi, p);
    const float z = __fsub_rn(t, s.hi);
    const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, z)), __fsub_rn(p, z));
    s.lo += err + e;
    s.hi = t;
}
__device__ __forceinline__ double df_value(DF s) { return f2d(s.hi) + f2d(s.lo); }

// Folded tile of an FP64 field as double-float pairs: [he][tc] even, [ho][tc] odd;
// each element float4 = (re.hi, re.lo, im.hi, im.lo).
// (skip0: mode 0 is left zero and not read, e.g. while another kernel writes it)
__device__ __forceinline__ void fold_load_df(float4* tile, const double2* __restrict__ src, const GridDev& g,
                                             int m0, int tc, int he, int ho, bool skip0 = false) {
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        double2 fe = make_double2(0.0, 0.0), fo = fe;
        if (m < g.nm && !(skip0 && m == 0)) {
            const double2 a = src[(size_t)k * g.nm + m];
            if (k < ho) {
                const double2 b = src[(size_t)(g.nz - 1 - k) * g.nm + m];
                fe = make_double2(a.x + b.x, a.y + b.y);
                fo = make_double2(a.x - b.x, a.y - b.y);
            } else {
                fe = a;
            }
        }
        const DF ex = df_split(fe.x), ey = df_split(fe.y);
        tile[t] = make_float4(ex.hi, ex.lo, ey.hi, ey.lo);
        if (k < ho) {
            const DF ox = df_split(fo.x), oy = df_split(fo.y);
            tile[(he + k) * tc + c] = make_float4(ox.hi, ox.lo, oy.hi, oy.lo);
        }
    }
}

// anti_apply_df's even and odd parts before their sum and difference:
// (ye.x, ye.y, yo.x, yo.y), yo zero at the unpaired mid level.
__device__ __forceinline__ double4 anti_apply_df_parts(const float2* __restrict__ De, const float2* __restrict__ Do,
                                                       const float4* tile, int k, int c, int tc, int he, int ho) {
    DF yex{0.f, 0.f}, yey{0.f, 0.f}, yox{0.f, 0.f}, yoy{0.f, 0.f};
    const float2* er = De + (size_t)k * ho;
    const float4* fo = tile + he * tc;
    for (int j = 0; j < ho; ++j) {
        const float2 a = __ldg(&er[j]);
        const float4 b = fo[j * tc + c];
        df_mac(yex, a.x, a.y, b.x, b.y);
        df_mac(yey, a.x, a.y, b.z, b.w);
    }
    if (k < ho) {
        const float2* orow = Do + (size_t)k * he;
        for (int j = 0; j < he; ++j) {
            const float2 a = __ldg(&orow[j]);
            const float4 b = tile[j * tc + c];
            df_mac(yox, a.x, a.y, b.x, b.y);
            df_mac(yoy, a.x, a.y, b.z, b.w);
        }
        return make_double4(df_value(yex), df_value(yey), df_value(yox), df_value(yoy));
    }
    return make_double4(df_value(yex), df_value(yey), 0.0, 0.0);
}

// Antisymmetric folded operator (double-float) on a double-float folded tile:
// the output pair (z = k, z = nz-1-k) as FP64.
__device__ __forceinline__ Pair anti_apply_df(const float2* __restrict__ De, const float2* __restrict__ Do,
                                              const float4* tile, int k, int c, int tc, int he, int ho) {
    const double4 y = anti_apply_df_parts(De, Do, tile, k, c, tc, he, ho);
    Pair p;
    p.a = make_double2(y.x + y.z, y.y + y.w);
    p.b = k < ho ? make_double2(y.x - y.z, y.y - y.w) : p.a;
    return p;
}

// Symmetric folded operator (double-float) on a double-float folded tile: the
// output pair (z = k, z = nz-1-k) as FP64 (sym_apply's fold).
__device__ __forceinline__ Pair sym_apply_df(const float2* __restrict__ Ae, const float2* __restrict__ Ao,
                                             const float4* tile, int k, int c, int tc, int he, int ho) {
    DF yex{0.f, 0.f}, yey{0.f, 0.f}, yox{0.f, 0.f}, yoy{0.f, 0.f};
    const float2* er = Ae + (size_t)k * he;
    for (int j = 0; j < he; ++j) {
        const float2 a = __ldg(&er[j]);
        const float4 b = tile[j * tc + c];
        df_mac(yex, a.x, a.y, b.x, b.y);
        df_mac(yey, a.x, a.y, b.z, b.w);
    }
    Pair p;
    if (k < ho) {
        const float2* orow = Ao + (size_t)k * ho;
        const float4* fo = tile + he * tc;
        for (int j = 0; j < ho; ++j) {
            const float2 a = __ldg(&orow[j]);
            const float4 b = fo[j * tc + c];
            df_mac(yox, a.x, a.y, b.x, b.y);
            df_mac(yoy, a.x, a.y, b.z, b.w);
        }
        const double ex = df_value(yex), ey = df_value(yey), ox = df_value(yox), oy = df_value(yoy);
        p.a = make_double2(ex + ox, ey + oy);
        p.b = make_double2(ex - ox, ey - oy);
    } else {
        p.a = make_double2(df_value(yex), df_value(yey));
        p.b = p.a;
    }
    return p;
}

// phi~_j = -(V'^T b)_j / (l'_j + k^2) of the folded right-hand sides tb of a
// mode tile, 4 eigen-rows of one block per thread, into tp.
__device__ __forceinline__ void pressure_mixed_forward(const GridDev& g, const MixedOps& mx, const Ops& ops,
                                                       const float* PAe, const float* PAo, const float2* tb,
                                                       float2* tp, int m0, int tc) {
    const int he = ops.he, ho = ops.ho;
    const int pe4 = mx.phe4, po4 = mx.pho4, nbe = pe4 / 4, nbo = po4 / 4;
    for (int t = threadIdx.x; t < (nbe + nbo) * tc; t += blockDim.x) {
        const int jb = t / tc, c = t - jb * tc;
        const int m = m0 + c;
        const bool even = jb < nbe;
        const int j0 = even ? 4 * jb : 4 * (jb - nbe);
        float2 acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = make_float2(0.f, 0.f);
        if (m < g.nm && m != 0) {
            const int len = even ? he : ho, ld4 = even ? nbe : nbo;
            const float4* __restrict__ A = reinterpret_cast<const float4*>(even ? PAe : PAo) + j0 / 4;
            const float2* b = tb + (even ? 0 : pe4 * tc) + c;
            for (int i = 0; i < len; ++i) {
                const float4 e = __ldg(&A[(size_t)i * ld4]);
                const float2 v = b[i * tc];
                acc[0].x = fmaf(e.x, v.x, acc[0].x); acc[0].y = fmaf(e.x, v.y, acc[0].y);
                acc[1].x = fmaf(e.y, v.x, acc[1].x); acc[1].y = fmaf(e.y, v.y, acc[1].y);
                acc[2].x = fmaf(e.z, v.x, acc[2].x); acc[2].y = fmaf(e.z, v.y, acc[2].y);
                acc[3].x = fmaf(e.w, v.x, acc[3].x); acc[3].y = fmaf(e.w, v.y, acc[3].y);
            }
            const int ky = m / g.nxhp, kx = m - ky * g.nxhp;
            const float k2 = d2f(__ldg(&ops.ksq[mode_q(ky, kx, g.ny, g.nxhp)]));
            const float* lam = even ? mx.plame : mx.plamo;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + q;
                const float sc = j < len ? -1.0f / (__ldg(&lam[j]) + k2) : 0.f;
                acc[q] = make_float2(sc * acc[q].x, sc * acc[q].y);
            }
        }
        float2* dst = tp + (even ? 0 : pe4 * tc) + c;
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[(j0 + q) * tc] = acc[q];
    }
}

// phi = pe + po, dphi/dz = dze + dzo at levels (i, nz-1-i) from tp, 4 rows i
// per thread: pe = PBe phi~e, po = PBo phi~o, dze = PDe phi~o, dzo = PDo
// phi~e; stored into PHI, PHIZ, or added to them (a correction).
template <bool kAdd>
__device__ __forceinline__ void pressure_mixed_back(const GridDev& g, const MixedOps& mx, const Ops& ops,
                                                    const float2* tp, double2* __restrict__ PHI,
                                                    double2* __restrict__ PHIZ, int m0, int tc) {
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    const int pe4 = mx.phe4, po4 = mx.pho4, nbe = pe4 / 4, nbo = po4 / 4;
    for (int t = threadIdx.x; t < nbe * tc; t += blockDim.x) {
        const int ib = t / tc, c = t - ib * tc;
        const int m = m0 + c;
        if (m >= g.nm || m == 0) continue;
        const int i0 = 4 * ib;
        float2 pe[4], po[4], de[4], dd[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { pe[q] = make_float2(0.f, 0.f); po[q] = pe[q]; de[q] = pe[q]; dd[q] = pe[q]; }
        const float2* qe = tp + c;
        const float2* qo = tp + pe4 * tc + c;
        {
            const float4* __restrict__ B = reinterpret_cast<const float4*>(mx.PBe) + ib;
            for (int j = 0; j < he; ++j) {
                const float4 a = __ldg(&B[(size_t)j * nbe]);
                const float2 v = qe[j * tc];
                pe[0].x = fmaf(a.x, v.x, pe[0].x); pe[0].y = fmaf(a.x, v.y, pe[0].y);
                pe[1].x = fmaf(a.y, v.x, pe[1].x); pe[1].y = fmaf(a.y, v.y, pe[1].y);
                pe[2].x = fmaf(a.z, v.x, pe[2].x); pe[2].y = fmaf(a.z, v.y, pe[2].y);
                pe[3].x = fmaf(a.w, v.x, pe[3].x); pe[3].y = fmaf(a.w, v.y, pe[3].y);
            }
            const float4* __restrict__ D = reinterpret_cast<const float4*>(mx.PDe) + ib;
            for (int j = 0; j < ho; ++j) {
                const float4 a = __ldg(&D[(size_t)j * nbe]);
                const float2 v = qo[j * tc];
                de[0].x = fmaf(a.x, v.x, de[0].x); de[0].y = fmaf(a.x, v.y, de[0].y);
                de[1].x = fmaf(a.y, v.x, de[1].x); de[1].y = fmaf(a.y, v.y, de[1].y);
                de[2].x = fmaf(a.z, v.x, de[2].x); de[2].y = fmaf(a.z, v.y, de[2].y);
                de[3].x = fmaf(a.w, v.x, de[3].x); de[3].y = fmaf(a.w, v.y, de[3].y);
            }
        }
        if (ib < nbo) {
            const float4* __restrict__ B = reinterpret_cast<const float4*>(mx.PBo) + ib;
            for (int j = 0; j < ho; ++j) {
                const float4 a = __ldg(&B[(size_t)j * nbo]);
                const float2 v = qo[j * tc];
                po[0].x = fmaf(a.x, v.x, po[0].x); po[0].y = fmaf(a.x, v.y, po[0].y);
                po[1].x = fmaf(a.y, v.x, po[1].x); po[1].y = fmaf(a.y, v.y, po[1].y);
                po[2].x = fmaf(a.z, v.x, po[2].x); po[2].y = fmaf(a.z, v.y, po[2].y);
                po[3].x = fmaf(a.w, v.x, po[3].x); po[3].y = fmaf(a.w, v.y, po[3].y);
            }
            const float4* __restrict__ D = reinterpret_cast<const float4*>(mx.PDo) + ib;
            for (int j = 0; j < he; ++j) {
                const float4 a = __ldg(&D[(size_t)j * nbo]);
                const float2 v = qe[j * tc];
                dd[0].x = fmaf(a.x, v.x, dd[0].x); dd[0].y = fmaf(a.x, v.y, dd[0].y);
                dd[1].x = fmaf(a.y, v.x, dd[1].x); dd[1].y = fmaf(a.y, v.y, dd[1].y);
                dd[2].x = fmaf(a.z, v.x, dd[2].x); dd[2].y = fmaf(a.z, v.y, dd[2].y);
                dd[3].x = fmaf(a.w, v.x, dd[3].x); dd[3].y = fmaf(a.w, v.y, dd[3].y);
            }
        }
        auto put = [&](size_t o, double2* F, float x, float y) {
            const double2 v = make_double2(f2d(x), f2d(y));
            if (kAdd) {
                const double2 o0 = F[o];
                F[o] = make_double2(o0.x + v.x, o0.y + v.y);
            } else {
                F[o] = v;
            }
        };
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + q;
            if (i >= he) break;
            const size_t o1 = (size_t)i * g.nm + m;
            if (i < ho) {
                const size_t o2 = (size_t)(nz - 1 - i) * g.nm + m;
                put(o1, PHI, pe[q].x + po[q].x, pe[q].y + po[q].y);
                put(o2, PHI, pe[q].x - po[q].x, pe[q].y - po[q].y);
                put(o1, PHIZ, de[q].x + dd[q].x, de[q].y + dd[q].y);
                put(o2, PHIZ, de[q].x - dd[q].x, de[q].y - dd[q].y);
            } else {
                put(o1, PHI, pe[q].x, pe[q].y);
                put(o1, PHIZ, de[q].x, de[q].y);
            }
        }
    }
}

// Pressure for the mixed form.  The right-hand side (the collocation
// divergence of u*, or the weak form) is formed in FP64: D applied to the
// full FP64 w* must not see FP32 rounding of w* (|D| ~ nz^2 would amplify it).
// The Neumann Poisson operator is diagonal in the eigenbasis of the full
// problem, S V' = M V' Lambda', V'^T M V' = I:
//   phi = -V' diag(1/(l'_j + k^2)) V'^T b,   dphi/dz = -(D V') diag(...) V'^T b
// evaluated in FP32 on the folded basis (even eigenvectors on the pair sums
// of b, odd ones on the differences, MixedOps); computing dphi/dz through the
// precomputed D V' keeps its FP32 error relative to dphi/dz itself.  Mode
// (0,0) (pinned) is left to the FP64 kernels.
// With sp.refine, one step of iterative refinement follows in the same CTA
// (each mode's system is its own): the residual r = b - P phi of the FP32
// solution, P = -S - diag(k^2 w ybar/2), is formed from the FP64 b and the
// stored phi with S applied in double-float (about 2^-48 relative, against
// the 2^-24 of the FP32 solve), and the FP32 solve of P d = r is added to
// phi and dphi/dz: the Galerkin residual drops from ~1e-7 to ~1e-13 of b.
template <bool kRefine>
__device__ __forceinline__ void pressure_mixed_body(GridDev g, MixedOps mx, Ops ops, StepParams sp,
                                                    const double2* __restrict__ US,
                                                    const double2* __restrict__ VS,
                                                    const double2* __restrict__ WS,
                                                    double2* __restrict__ PHI, double2* __restrict__ PHIZ,
                                                    int tc, int bx) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nz = g.nz, he = ops.he, ho = ops.ho;
    const int pe4 = mx.phe4, po4 = mx.pho4;
    float4* tw = reinterpret_cast<float4*>(smraw);              // folded w* (double-float)  [nz][tc]
    float2* tb = reinterpret_cast<float2*>(tw + nz * tc);       // folded rhs: s [pe4][tc], d [po4][tc]
    float2* tp = tb + (pe4 + po4) * tc;                         // phi~: even [pe4][tc], odd [po4][tc]
    double2* bt = reinterpret_cast<double2*>(tp + (pe4 + po4) * tc);  // FP64 rhs [nz][tc] (refinement)
    const int m0 = bx * tc;
    fold_load_df(tw, WS, g, m0, tc, he, ho);
    for (int t = threadIdx.x; t < (pe4 - he) * tc; t += blockDim.x) tb[he * tc + t] = make_float2(0.f, 0.f);
    for (int t = threadIdx.x; t < (po4 - ho) * tc; t += blockDim.x) tb[(pe4 + ho) * tc + t] = make_float2(0.f, 0.f);
    __syncthreads();
    const float2* __restrict__ Ae = sp.weak_form ? mx.W1e_df : mx.D1e_df;
    const float2* __restrict__ Ao = sp.weak_form ? mx.W1o_df : mx.D1o_df;
    // right-hand side pair (k, nz-1-k), folded in FP64 before the rounding
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        float2 fs = make_float2(0.f, 0.f), fd = fs;
        double2 b1 = make_double2(0.0, 0.0), b2 = b1;
        if (m < g.nm && m != 0) {
            const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
            if (!kRefine && !sp.weak_form) {
                // the folded strong-form right-hand side divided by 2 w_k / dt
                // (the scaled forward operators PAeS, PAoS carry that factor):
                // (b_k +- b_k') dt / (2 w_k) = i (ax/2)(u_k +- u_k') +
                // i (ay/2)(v_k +- v_k') + (ye | yo), the mid level
                // i (ax/2) u_k + i (ay/2) v_k + ye / 2; ye, yo the even and
                // odd parts of D1.w* -- 20 FP64 operations per level pair
                // instead of 36
                const double4 y = anti_apply_df_parts(Ae, Ao, tw, k, c, tc, he, ho);
                const double hax = 0.5 * mi.ax, hay = 0.5 * mi.ay;
                const size_t o1 = (size_t)k * g.nm + m;
                const double2 u1 = US[o1], v1 = VS[o1];
                if (k < ho) {
                    const size_t o2 = (size_t)(nz - 1 - k) * g.nm + m;
                    const double2 u2 = US[o2], v2 = VS[o2];
                    const double2 up = make_double2(u1.x + u2.x, u1.y + u2.y), um = make_double2(u1.x - u2.x, u1.y - u2.y);
                    const double2 vp = make_double2(v1.x + v2.x, v1.y + v2.y), vm = make_double2(v1.x - v2.x, v1.y - v2.y);
                    fs = make_float2(d2f(fma(-hax, up.y, fma(-hay, vp.y, y.x))), d2f(fma(hax, up.x, fma(hay, vp.x, y.y))));
                    fd = make_float2(d2f(fma(-hax, um.y, fma(-hay, vm.y, y.z))), d2f(fma(hax, um.x, fma(hay, vm.x, y.w))));
                } else {
                    fs = make_float2(d2f(fma(-hax, u1.y, fma(-hay, v1.y, 0.5 * y.x))),
                                     d2f(fma(hax, u1.x, fma(hay, v1.x, 0.5 * y.y))));
                }
            } else {
                const Pair dz = anti_apply_df(Ae, Ao, tw, k, c, tc, he, ho);
                b1 = pressure_rhs(g, ops, sp, k, m, mi, US, VS, dz.a);
                if (k < ho) {
                    b2 = pressure_rhs(g, ops, sp, nz - 1 - k, m, mi, US, VS, dz.b);
                    fs = make_float2(d2f(b1.x + b2.x), d2f(b1.y + b2.y));
                    fd = make_float2(d2f(b1.x - b2.x), d2f(b1.y - b2.y));
                } else {
                    fs = make_float2(d2f(b1.x), d2f(b1.y));
                }
            }
        }
        tb[k * tc + c] = fs;
        if (k < ho) tb[(pe4 + k) * tc + c] = fd;
        if (kRefine) {
            bt[k * tc + c] = b1;
            if (k < ho) bt[(nz - 1 - k) * tc + c] = b2;
        }
    }
    __syncthreads();
    const bool scaled = !kRefine && !sp.weak_form;
    pressure_mixed_forward(g, mx, ops, scaled ? mx.PAeS : mx.PAe, scaled ? mx.PAoS : mx.PAo, tb, tp, m0, tc);
    __syncthreads();
    pressure_mixed_back<false>(g, mx, ops, tp, PHI, PHIZ, m0, tc);
    if (!kRefine) return;
    // refinement: r = b + S phi + k^2 wh phi (phi as stored, FP64)
    __syncthreads();  // this CTA's PHI writes, then the folded phi in double-float
    fold_load_df(tw, PHI, g, m0, tc, he, ho, true);
    __syncthreads();
    for (int t = threadIdx.x; t < he * tc; t += blockDim.x) {
        const int k = t / tc, c = t - k * tc;
        const int m = m0 + c;
        float2 fs = make_float2(0.f, 0.f), fd = fs;
        if (m < g.nm && m != 0) {
            const Pair sphi = sym_apply_df(mx.Se_df, mx.So_df, tw, k, c, tc, he, ho);
            const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
            const double k2 = __ldg(&ops.ksq[mode_q(mi.ky, mi.kx, g.ny, g.nxhp)]);
            const double2 p1 = PHI[(size_t)k * g.nm + m], c1 = bt[k * tc + c];
            const double kw1 = k2 * __ldg(&ops.wh[k]);
            const double2 r1 = make_double2(c1.x + sphi.a.x + kw1 * p1.x, c1.y + sphi.a.y + kw1 * p1.y);
            if (k < ho) {
                const double2 p2 = PHI[(size_t)(nz - 1 - k) * g.nm + m], c2 = bt[(nz - 1 - k) * tc + c];
                const double kw2 = k2 * __ldg(&ops.wh[nz - 1 - k]);
                const double2 r2 = make_double2(c2.x + sphi.b.x + kw2 * p2.x, c2.y + sphi.b.y + kw2 * p2.y);
                fs = make_float2(d2f(r1.x + r2.x), d2f(r1.y + r2.y));
                fd = make_float2(d2f(r1.x - r2.x), d2f(r1.y - r2.y));
            } else {
                fs = make_float2(d2f(r1.x), d2f(r1.y));
            }
        }
        tb[k * tc + c] = fs;
        if (k < ho) tb[(pe4 + k) * tc + c] = fd;
    }
    __syncthreads();
    pressure_mixed_forward(g, mx, ops, mx.PAe, mx.PAo, tb, tp, m0, tc);
    __syncthreads();
    pressure_mixed_back<true>(g, mx, ops, tp, PHI, PHIZ, m0, tc);
}

template <bool kRefine>
__global__ void __launch_bounds__(256) k_pressure_mixed(GridDev g, MixedOps mx, Ops ops, StepParams sp,
                                                        const double2* __restrict__ US,
                                                        const double2* __restrict__ VS,
                                                        const double2* __restrict__ WS,
                                                        double2* __restrict__ PHI, double2* __restrict__ PHIZ,
                                                        int tc) {
    pressure_mixed_body<kRefine>(g, mx, ops, sp, US, VS, WS, PHI, PHIZ, tc, blockIdx.x);
}

// dphi/dz of mode (0,0) in FP64 (one CTA), after k_pressure has written phi.
__device__ __forceinline__ void dz_mean_mode_body(GridDev g, Ops ops, const double2* __restrict__ PHI,
                                                  double2* __restrict__ PHIZ, int bx) {
    extern __shared__ double2 sm[];
    const int he = ops.he, ho = ops.ho;
    fold_load(sm, PHI, g, 0, 1, he, ho);
    __syncthreads();
    for (int k = threadIdx.x; k < he; k += blockDim.x) {
        const Pair d = anti_apply(ops.D1e, ops.D1o, sm, k, 0, 1, he, ho);
        PHIZ[(size_t)k * g.nm] = d.a;
        if (k < ho) PHIZ[(size_t)(g.nz - 1 - k) * g.nm] = d.b;
    }
}

__global__ void __launch_bounds__(256) k_dz_mean_mode(GridDev g, Ops ops, const double2* __restrict__ PHI,
                                                      double2* __restrict__ PHIZ) {
    dz_mean_mode_body(g, ops, PHI, PHIZ, blockIdx.x);
}

// Pointwise correction of the mixed form (pressure_correction_3d, 3D:1903-1929)
// with dphi/dz precomputed: u = u* - dt DX phi, v = v* - dt DY phi,
// w = w* - dt dphi/dz, p += phi, wall gradients of the new p.
__device__ __forceinline__ void correction_mixed_body(GridDev g, Ops ops, StepParams sp, const double2* __restrict__ US,
                                                      const double2* __restrict__ VS, const double2* __restrict__ WS,
                                                      const double2* __restrict__ PHI, const double2* __restrict__ PHIZ,
                                                      double2* __restrict__ U, double2* __restrict__ V, double2* __restrict__ W,
                                                      double2* __restrict__ P, double2* __restrict__ GP, int bx, int gx) {
    const size_t n = (size_t)g.nz * g.nm;
    const size_t stride = (size_t)gx * blockDim.x;
    const double dt = sp.dt;
    for (size_t o = (size_t)bx * blockDim.x + threadIdx.x; o < n; o += stride) {
        const int z = (int)(o / g.nm);
        const int m = (int)(o - (size_t)z * g.nm);
        const ModeInfo mi = mode_info(g, m, ops.xw, ops.yw);
        const double dax = dt * mi.ax, day = dt * mi.ay;
        const double2 ph = PHI[o], pz = PHIZ[o];
        const double2 us = US[o], vs = VS[o], ws = WS[o];
        // u* - dt (i ax) phi, v* - dt (i ay) phi, w* - dt dphi/dz with fused products
        store_projection(sp, z, g.nz, o, make_double2(fma(dax, ph.y, us.x), fma(-dax, ph.x, us.y)),
                         make_double2(fma(day, ph.y, vs.x), fma(-day, ph.x, vs.y)),
                         make_double2(fma(-dt, pz.x, ws.x), fma(-dt, pz.y, ws.y)), U, V, W);
        double2 pp = P[o];
        pp.x += ph.x;
        pp.y += ph.y;
        P[o] = pp;
        if (z == 0 || z == g.nz - 1) {
            const int wall = (z == 0) ? 0 : 1;
            GP[(size_t)wall * g.nm + m] = i_times(mi.ax, pp);
            GP[(size_t)(2 + wall) * g.nm + m] = i_times(mi.ay, pp);
        }
    }
}

__global__ void k_correction_mixed(GridDev g, Ops ops, StepParams sp, const double2* __restrict__ US,
                                   const double2* __restrict__ VS, const double2* __restrict__ WS,
                                   const double2* __restrict__ PHI, const double2* __restrict__ PHIZ,
                                   double2* __restrict__ U, double2* __restrict__ V, double2* __restrict__ W,
                                   double2* __restrict__ P, double2* __restrict__ GP) {
    correction_mixed_body(g, ops, sp, US, VS, WS, PHI, PHIZ, U, V, W, P, GP, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ reductions

// Per-block partials of max|u|, max|v|, max|w| and sum 0.5|u|^2 zwts[k].
// Block (bx, k) reduces part bx of plane k: max |u|, |v|, |w| as the largest
// bit pattern of |x| (integer comparisons order non-negative doubles, and a
// NaN beats every number), and the plane's sum of |u|^2 scaled by 0.5 w_k once.
__global__ void __launch_bounds__(256) k_diag_partial(GridDev g, const double* __restrict__ zw,
                                                      const double* __restrict__ u,
                                                      const double* __restrict__ v,
                                                      const double* __restrict__ w,
                                                      double* __restrict__ partial) {
    const size_t plane = (size_t)g.nx * g.ny;
    const size_t off = (size_t)blockIdx.y * plane;
    const unsigned long long am = 0x7FFFFFFFFFFFFFFFULL;
    unsigned long long mu = 0, mv = 0, mw = 0;
    double e = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
        const double a = u[off + i], b = v[off + i], c = w[off + i];
        mu = max(mu, (unsigned long long)__double_as_longlong(a) & am);
        mv = max(mv, (unsigned long long)__double_as_longlong(b) & am);
        mw = max(mw, (unsigned long long)__double_as_longlong(c) & am);
        e = fma(a, a, e);
        e = fma(b, b, e);
        e = fma(c, c, e);
    }
    __shared__ unsigned long long redm[3][8];
    __shared__ double rede[8];
    for (int o = 16; o > 0; o >>= 1) {
        mu = max(mu, __shfl_xor_sync(0xffffffffu, mu, o));
        mv = max(mv, __shfl_xor_sync(0xffffffffu, mv, o));
        mw = max(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    }
    e = warp_sum(e);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { redm[0][wid] = mu; redm[1][wid] = mv; redm[2][wid] = mw; rede[wid] = e; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            mu = max(mu, redm[0][k]); mv = max(mv, redm[1][k]); mw = max(mw, redm[2][k]); e += rede[k];
        }
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
        partial[4 * b + 0] = __longlong_as_double((long long)mu);
        partial[4 * b + 1] = __longlong_as_double((long long)mv);
        partial[4 * b + 2] = __longlong_as_double((long long)mw);
        partial[4 * b + 3] = 0.5 * e * __ldg(&zw[blockIdx.y]);
    }
}

// One warp: lane l folds partials l, l+32, ...; then a butterfly.
__device__ __forceinline__ unsigned long long bits_of(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void k_diag_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    unsigned long long mu = 0, mv = 0, mw = 0;  // |x| bit patterns (NaN beats every number)
    double e = 0.0;
    for (int b = threadIdx.x; b < nb; b += 32) {
        mu = max(mu, bits_of(partial[4 * b]));
        mv = max(mv, bits_of(partial[4 * b + 1]));
        mw = max(mw, bits_of(partial[4 * b + 2]));
        e += partial[4 * b + 3];
    }
    mu = warp_max_bits(mu); mv = warp_max_bits(mv); mw = warp_max_bits(mw); e = warp_sum(e);
    if (threadIdx.x == 0) {
        out[0] = __longlong_as_double((long long)mu);
        out[1] = __longlong_as_double((long long)mv);
        out[2] = __longlong_as_double((long long)mw);
        out[3] = e;
    }
}

// The controller state and the (0,0) mode of u, v, w per level, gathered
// next to the reductions so that one copy brings all diagnostics back.
__global__ void k_diag_gather(GridDev g, const double2* __restrict__ U, const double2* __restrict__ V,
                              const double2* __restrict__ W, const dns3d_pi_state* __restrict__ pi,
                              double* __restrict__ out) {
    const double* ps = reinterpret_cast<const double*>(pi);
    constexpr int npi = (int)(sizeof(dns3d_pi_state) / sizeof(double));
    for (int t = threadIdx.x; t < npi; t += blockDim.x) out[t] = ps[t];
    double2* mean = reinterpret_cast<double2*>(out + npi);
    const double2* f[3] = {U, V, W};
    for (int t = threadIdx.x; t < 3 * g.nz; t += blockDim.x) {
        const int c = t / g.nz, k = t - c * g.nz;
        mean[t] = f[c][(size_t)k * g.nm];
    }
}

// max |f| as the largest bit pattern of |f| (integer comparisons; a NaN wins)
__global__ void __launch_bounds__(256) k_maxabs_partial(const double* __restrict__ f, size_t n,
                                                        double* __restrict__ partial) {
    unsigned long long m = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        m = max(m, bits_of(f[i]) & 0x7FFFFFFFFFFFFFFFULL);
    __shared__ unsigned long long red[8];
    m = warp_max_bits(m);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) m = max(m, red[k]);
        partial[blockIdx.x] = __longlong_as_double((long long)m);
    }
}

__global__ void k_max_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    unsigned long long m = 0;
    for (int b = threadIdx.x; b < nb; b += 32) m = max(m, bits_of(partial[b]));
    m = warp_max_bits(m);
    if (threadIdx.x == 0) out[0] = __longlong_as_double((long long)m);
}

__global__ void k_nonfinite(const double2* __restrict__ f, size_t n, int* flag) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    int bad = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double2 a = f[i];
        if (!isfinite(a.x) || !isfinite(a.y)) bad = 1;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

int tile_cols(const GridDev& g, int narrays) {
    // Largest TC in {32,16,8,4} whose tiles fit ~96 KB and that still gives
    // at least two CTAs per SM on 152 SMs; never below 4.
    int tc = 32;
    while (tc > 4 && ((size_t)narrays * g.nz * tc * sizeof(double2) > 96 * 1024 ||
                      (g.nm + tc - 1) / tc < 304))
        tc >>= 1;
    return tc;
}

// The dynamic shared-memory limit is a property of the kernel function, shared
// by every handle in the process, so it is raised to the device's opt-in
// maximum rather than to one grid's need (a smaller grid's handle would
// otherwise lower it below what a larger grid's launches request).
template <typename K>
cudaError_t set_smem(K kern, size_t bytes) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev))) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, kern))) return e;
    const int limit = optin - (int)fa.sharedSizeBytes;  // static + dynamic <= opt-in maximum
    if (bytes > (size_t)limit) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
}

}  // namespace

int pad4(int n) { return (n + 3) / 4 * 4; }

size_t viscous_mixed_smem(const GridDev& g, int tc) {
    const size_t ni = g.nz - 2, hoi = ni / 2, hei = ni - hoi, pe4 = pad4((int)hei), po4 = pad4((int)hoi);
    return 2 * (hei * pe4 + hoi * po4) * sizeof(float) + 3 * (pe4 + po4) * tc * sizeof(float2) +
           tc * (sizeof(float4) + sizeof(float));
}

int tile_cols_mixed(const GridDev& g) {
    int tc = 32;
    while (tc > 4 && (viscous_mixed_smem(g, tc) > 110 * 1024 || (g.nm + tc - 1) / tc < 152)) tc >>= 1;
    return tc;
}

size_t pressure_mixed_smem(const GridDev& g, int tc) {
    const int ho = g.nz / 2, he = g.nz - ho;
    return (size_t)g.nz * tc * sizeof(float4) + 2 * (size_t)(pad4(he) + pad4(ho)) * tc * sizeof(float2) +
           (g.refine ? (size_t)g.nz * tc * sizeof(double2) : 0);  // the FP64 right-hand side kept for the refinement
}

namespace {

size_t tile_smem(const GridDev& g, int k, int tc) {
    const size_t nz = g.nz;
    switch (k) {
        case kTileVort: return 2 * nz * tc * sizeof(double2);
        case kTileVisc: return 6 * nz * tc * sizeof(double2);
        case kTilePres: return (2 * nz * tc + nz) * sizeof(double2);
        case kTileCorr: return nz * tc * sizeof(double2);
        case kTileDiv: return nz * tc * sizeof(double2);
        case kTileVortM: return 2 * nz * tc * sizeof(float2);
        case kTileViscM: return viscous_mixed_smem(g, tc);
        case kTilePresM: return pressure_mixed_smem(g, tc);
    }
    return 0;
}

template <typename K>
size_t smem_limit(K kern) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return 0;
    return (size_t)fa.maxDynamicSharedSizeBytes;
}

}  // namespace

int tile_width(const GridDev& g, int k) {
    if (k >= 0 && k < kTileKernels && g.tc[k] > 0) return g.tc[k];
    switch (k) {
        case kTileVort: return tile_cols(g, 2);
        case kTileVisc: return tile_cols(g, 6);
        case kTilePres: return tile_cols(g, 2);
        case kTileCorr: return tile_cols(g, 1);
        case kTileDiv: return tile_cols(g, 1);
        case kTileVortM: return tile_cols(g, 1);
        case kTileViscM: return tile_cols_mixed(g);
        case kTilePresM: return tile_cols(g, 2);
    }
    return 8;
}

bool tile_fits(const GridDev& g, int k, int tc) {
    if (tc < 1) return false;
    size_t lim = 0;
    switch (k) {
        case kTileVort: lim = smem_limit(k_vorticity); break;
        case kTileVisc: lim = smem_limit(k_viscous<double2>); break;
        case kTilePres: lim = smem_limit(k_pressure); break;
        case kTileCorr: lim = smem_limit(k_correction); break;
        case kTileDiv: lim = smem_limit(k_divergence); break;
        case kTileVortM: lim = smem_limit(k_vorticity_mixed); break;
        case kTileViscM: lim = smem_limit(k_viscous_mixed); break;
        case kTilePresM: lim = std::min(smem_limit(k_pressure_mixed<false>), smem_limit(k_pressure_mixed<true>)); break;
        default: return false;
    }
    return tile_smem(g, k, tc) <= lim;
}

cudaError_t prepare_step_kernels(const GridDev& g) {
    cudaError_t e;
    if ((e = set_smem(k_pressure, (2 * (size_t)g.nz + g.nz) * sizeof(double2)))) return e;
    if ((e = set_smem(k_correction, (size_t)g.nz * sizeof(double2)))) return e;
    if ((e = set_smem(k_pressure_mixed<false>, pressure_mixed_smem(g, tile_cols(g, 2))))) return e;
    if ((e = set_smem(k_pressure_mixed<true>, pressure_mixed_smem(g, tile_cols(g, 2))))) return e;
    if ((e = set_smem(k_viscous<float2>, 6 * (size_t)g.nz * sizeof(double2)))) return e;
    if ((e = set_smem(k_vorticity_mixed, 2 * (size_t)g.nz * tile_cols(g, 1) * sizeof(float2)))) return e;
    if ((e = set_smem(k_viscous_mixed, viscous_mixed_smem(g, tile_cols_mixed(g))))) return e;
    if ((e = set_smem(k_vorticity, 2 * (size_t)g.nz * tile_cols(g, 2) * sizeof(double2)))) return e;
    if ((e = set_smem(k_viscous<double2>, 6 * (size_t)g.nz * tile_cols(g, 6) * sizeof(double2)))) return e;
    if ((e = set_smem(k_pressure, (2 * (size_t)g.nz * tile_cols(g, 2) + g.nz) * sizeof(double2)))) return e;
    if ((e = set_smem(k_correction, (size_t)g.nz * tile_cols(g, 1) * sizeof(double2)))) return e;
    if ((e = set_smem(k_divergence, (size_t)g.nz * tile_cols(g, 1) * sizeof(double2)))) return e;
    if ((e = set_smem(k_viscous_tc<false>, 0))) return e;
    if ((e = set_smem(k_viscous_tc<true>, 0))) return e;
    if ((e = set_smem(k_dz_tc<VortTcOp>, 0))) return e;
    if ((e = set_smem(k_dz_tc<CorrTcOp>, 0))) return e;
    if ((e = set_smem(k_dz_tc<PresRhsTcOp>, 0))) return e;
    if ((e = set_smem(k_pressure_solve, 0))) return e;
    if ((e = set_smem(k_pcg_poisson, pcg_smem(g)))) return e;
    if ((e = set_smem(k_pcg_helmholtz, pcg_smem(g)))) return e;
    return cudaSuccess;
}

namespace {
// d2f / f2d (cvt.cuh) against the hardware conversions on n doubles spread
// over the normal float range (SplitMix64 bits: sign, exponent in
// [-126, 127], all mantissas), and on every float of a strided sweep for f2d;
// i2d_scaled against the hardware int64 -> FP64 conversion and ldexp.
__global__ void k_cvt_check(long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long nb = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + (unsigned long long)i * 0x9E3779B97F4A7C15ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        const unsigned long long e = 1023 - 126 + (z >> 52) % 254;  // float exponents -126 .. 127
        const double x = __longlong_as_double((long long)((z & 0x800FFFFFFFFFFFFFULL) | (e << 52)));
        if (__float_as_uint(d2f(x)) != __float_as_uint(__double2float_rn(x))) ++nb;
        const float v = __uint_as_float((unsigned)(z >> 32));
        if (isfinite(v) && __double_as_longlong(f2d(v)) != __double_as_longlong((double)v)) ++nb;
        // i2d_scaled: integers of every bit length, scalings into and out of the normal range
        const long long X = (long long)(z * 0xD1B54A32D192ED03ULL) >> (int)(z & 63);
        const int e2 = (int)((z >> 8) % 2200) - 1150;
        if (__double_as_longlong(i2d_scaled(X, e2)) != __double_as_longlong(ldexp(__ll2double_rn(X), e2))) ++nb;
    }
    if (nb) atomicAdd(bad, nb);
}
}  // namespace

cudaError_t check_conversions(long long n, unsigned long long* mismatches) {
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
    if (e) return e;
    cudaMemset(d, 0, sizeof(unsigned long long));
    k_cvt_check<<<152 * 8, 256>>>(n, 0x5DEECE66DULL, d);
    e = cudaMemcpy(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

cudaError_t launch_pi_update(const GridDev& g, const Ops& ops, const PIParams& pp, const double2* U,
                             dns3d_pi_state* pi, cudaStream_t s) {
    k_pi_update<<<1, 128, 0, s>>>(g, ops.zw, pp, U, pi);
    return cudaGetLastError();
}

cudaError_t launch_vorticity(const GridDev& g, const Ops& ops, const double2* U, const double2* V,
                             const double2* W, double2* OX, double2* OY, double2* OZ, cudaStream_t s) {
    const int tc = tile_width(g, kTileVort);
    const size_t sm = 2 * (size_t)g.nz * tc * sizeof(double2);
    k_vorticity<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, U, V, W, OX, OY, OZ, tc);
    return cudaGetLastError();
}

cudaError_t launch_products(const GridDev& g, RFields in6, RFields out3, cudaStream_t s) {
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_products<<<blocks, 256, 0, s>>>(in6, out3, n);
    return cudaGetLastError();
}

cudaError_t launch_viscous(const GridDev& g, const Ops& ops, const StepParams& sp, Fields F,
                           Fields Src, const double2* GP, const dns3d_pi_state* pi, Fields Out,
                           cudaStream_t s) {
    const int tc = tile_width(g, kTileVisc);
    const size_t sm = 6 * (size_t)g.nz * tc * sizeof(double2);
    k_viscous<double2><<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, sp, F, Src, GP, pi, Out, tc);
    return cudaGetLastError();
}

cudaError_t launch_poisson_residual(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                    const double2* VS, const double2* WS, const double2* PHI,
                                    unsigned long long* out, cudaStream_t s) {
    constexpr int tc = 16;
    const size_t sm = 2 * (size_t)g.nz * tc * sizeof(double2);
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if ((e = set_smem(k_poisson_residual, sm)) != cudaSuccess) return e;
    k_poisson_residual<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, sp, US, VS, WS, PHI, tc, out);
    return cudaGetLastError();
}

size_t viscous_tc_smem(const GridDev& g) {
    // + the staged inputs where they fit
    return viscous_tc_pipelined(g.nz) ? viscous_tc_smem_nz<true>(g.nz) : viscous_tc_smem_nz<false>(g.nz);
}

// Streaming multiprocessors of the current device (read once per device).
int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

bool viscous_tc_fits(const GridDev& g) {
    return tc_supported(g.nz) &&
           viscous_tc_smem(g) <= (viscous_tc_pipelined(g.nz) ? smem_limit(k_viscous_tc<true>)
                                                             : smem_limit(k_viscous_tc<false>));
}

// Operator indices q per CTA: consecutive runs of q spread over one wave of
// CTAs (two on each of 152 SMs), so every CTA stages its next q's inputs while
// it works on the current one and no partial wave is left at the end; a CTA's
// consecutive q (neighbouring kx) share cache sectors.  Which CTA takes a q
// does not change its arithmetic.
int tc_q_per_cta(int nq) { return std::max(1, (nq + 2 * 152 - 1) / (2 * 152)); }

cudaError_t launch_viscous_tc(const GridDev& g, const Ops& ops, const StepParams& sp, Fields F, Fields Src,
                              const double2* GP, const dns3d_pi_state* pi, Fields Out, int* err, cudaStream_t s) {
    if (!ops.tcA || !ops.tcE || !viscous_tc_fits(g)) return cudaErrorInvalidValue;
    const int qpb = tc_q_per_cta(ops.nq);
    const int nb = (ops.nq + qpb - 1) / qpb;
    if (viscous_tc_pipelined(g.nz))
        k_viscous_tc<true><<<nb, 256, viscous_tc_smem(g), s>>>(g, ops, sp, F, Src, GP, pi, Out, qpb, err);
    else
        k_viscous_tc<false><<<nb, 256, viscous_tc_smem(g), s>>>(g, ops, sp, F, Src, GP, pi, Out, qpb, err);
    return cudaGetLastError();
}

size_t vorticity_tc_smem(const GridDev& g) {
    const TcGeom t = tc_geom(g.nz);
    return dz_tc_stage_offset(t) + (dz_tc_staged(t, g.nz) ? (size_t)(kTcVortCols / 2) * g.nz * sizeof(double2) : 0);
}

bool vorticity_tc_fits(const GridDev& g) {
    return tc_supported(g.nz) && vorticity_tc_smem(g) <= smem_limit(k_dz_tc<VortTcOp>) &&
           vorticity_tc_smem(g) <= smem_limit(k_dz_tc<CorrTcOp>) &&
           vorticity_tc_smem(g) <= smem_limit(k_dz_tc<PresRhsTcOp>);
}

// Tiles (of `modes` modes) per CTA: at least 4 (the D1 image is copied once
// per CTA), else two CTAs per SM.  The chunking does not change a tile's
// arithmetic.
int tc_dz_chunk(int nm, int modes) {
    const int ntiles = (nm + modes - 1) / modes;
    return std::max(4, (ntiles + 2 * 152 - 1) / (2 * 152));
}

template <class Op>
cudaError_t launch_dz_tc(const GridDev& g, const Ops& ops, const Op& op, int* err, cudaStream_t s) {
    if (!ops.tcD || !ops.tcDE || !vorticity_tc_fits(g)) return cudaErrorInvalidValue;
    constexpr int kModes = kTcVortCols / (2 * Op::kFields);
    const int ntiles = (g.nm + kModes - 1) / kModes;
    const int chunk = tc_dz_chunk(g.nm, kModes);
    k_dz_tc<Op><<<(ntiles + chunk - 1) / chunk, kTcVortThreads, vorticity_tc_smem(g), s>>>(g, ops, op, chunk, err);
    return cudaGetLastError();
}

cudaError_t launch_vorticity_tc(const GridDev& g, const Ops& ops, const double2* U, const double2* V,
                                const double2* W, double2* OX, double2* OY, double2* OZ, int* err, cudaStream_t s) {
    const VortTcOp op{U, V, W, OX, OY, OZ};
    return launch_dz_tc(g, ops, op, err, s);
}

cudaError_t launch_pressure_tc(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                               const double2* VS, const double2* WS, double2* PHI, int* err, cudaStream_t s) {
    // the weak form's operator has no digit image; the solve needs the fixed-point inverses
    if (sp.weak_form || !ops.PinvI) return cudaErrorInvalidValue;
    const PresRhsTcOp op{sp, US, VS, WS, PHI};
    cudaError_t e = launch_dz_tc(g, ops, op, err, s);
    if (e) return e;
    const int tc = fx_solve_modes(g.nz);
    k_pressure_solve<<<(g.nm + tc - 1) / tc, fx_solve_threads(g.nz), fx_solve_smem(g.nz), s>>>(g, ops, PHI);
    return cudaGetLastError();
}

cudaError_t launch_correction_tc(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                 const double2* VS, const double2* WS, const double2* PHI, double2* U, double2* V,
                                 double2* W, double2* P, double2* GP, int* err, cudaStream_t s) {
    const CorrTcOp op{sp, US, VS, WS, PHI, U, V, W, P, GP};
    return launch_dz_tc(g, ops, op, err, s);
}

cudaError_t launch_vorticity_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops, const double2* U,
                                   const double2* V, const double2* W, FFields out, cudaStream_t s) {
    const int tc = tile_width(g, kTileVortM);
    const size_t sm = 2 * (size_t)g.nz * tc * sizeof(float2);
    k_vorticity_mixed<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, mx, ops, U, V, W, out, tc);
    return cudaGetLastError();
}

cudaError_t launch_pressure_mean_mode(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                      const double2* VS, const double2* WS, double2* PHI, double2* PHIZ,
                                      cudaStream_t s) {
    // mode (0,0) of the mixed form in FP64: pinned Poisson, then its dphi/dz
    k_pressure<<<1, 256, (2 * (size_t)g.nz + g.nz) * sizeof(double2), s>>>(g, ops, sp, US, VS, WS, PHI, 1);
    k_dz_mean_mode<<<1, 64, (size_t)g.nz * sizeof(double2), s>>>(g, ops, PHI, PHIZ);
    return cudaGetLastError();
}

cudaError_t launch_pressure_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops, const StepParams& sp,
                                  const double2* US, const double2* VS, const double2* WS, double2* PHI,
                                  double2* PHIZ, cudaStream_t s) {
    const int tc = tile_width(g, kTilePresM);
    const size_t sm = pressure_mixed_smem(g, tc);
    if (sp.refine)
        k_pressure_mixed<true><<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, mx, ops, sp, US, VS, WS, PHI, PHIZ, tc);
    else
        k_pressure_mixed<false><<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, mx, ops, sp, US, VS, WS, PHI, PHIZ, tc);
    return cudaGetLastError();
}

cudaError_t launch_correction_mixed(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                                    const double2* VS, const double2* WS, const double2* PHI, const double2* PHIZ,
                                    double2* U, double2* V, double2* W, double2* P, double2* GP, cudaStream_t s) {
    const size_t n = (size_t)g.nz * g.nm;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_correction_mixed<<<blocks, 256, 0, s>>>(g, ops, sp, US, VS, WS, PHI, PHIZ, U, V, W, P, GP);
    return cudaGetLastError();
}

cudaError_t launch_products32(const GridDev& g, FRFields in6, FRFields out3, cudaStream_t s) {
    const size_t n = (size_t)g.nx * g.ny * g.nz;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_products32<<<blocks, 256, 0, s>>>(in6, out3, n);
    return cudaGetLastError();
}

cudaError_t launch_viscous_mean_mode(const GridDev& g, const Ops& ops, const StepParams& sp, Fields F, FFields Src,
                                     const double2* GP, const dns3d_pi_state* pi, Fields Out, cudaStream_t s) {
    // mode (0,0) of the mixed form: FP64 Helmholtz with the forcing (one CTA)
    k_viscous<float2><<<1, 256, 6 * (size_t)g.nz * sizeof(double2), s>>>(g, ops, sp, F, Src, GP, pi, Out, 1);
    return cudaGetLastError();
}

cudaError_t launch_viscous_mixed(const GridDev& g, const MixedOps& mx, const Ops& ops, const StepParams& sp,
                                 Fields F, FFields Src, const double2* GP, Fields Out, cudaStream_t s) {
    const int tc = tile_width(g, kTileViscM);
    const size_t sm = viscous_mixed_smem(g, tc);
    const int ntiles = (g.nm + tc - 1) / tc;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_viscous_mixed, 256, sm);
    if (e) return e;
    const int nb = std::min(ntiles, std::max(1, per_sm) * num_sms());
    k_viscous_mixed<<<nb, 256, sm, s>>>(g, mx, ops, sp, F, Src, GP, Out, tc);
    return cudaGetLastError();
}

cudaError_t launch_pressure(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                            const double2* VS, const double2* WS, double2* PHI, cudaStream_t s) {
    const int tc = tile_width(g, kTilePres);
    const size_t sm = (2 * (size_t)g.nz * tc + g.nz) * sizeof(double2);
    k_pressure<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, sp, US, VS, WS, PHI, tc);
    return cudaGetLastError();
}

cudaError_t launch_correction(const GridDev& g, const Ops& ops, const StepParams& sp, const double2* US,
                              const double2* VS, const double2* WS, const double2* PHI, double2* U,
                              double2* V, double2* W, double2* P, double2* GP, cudaStream_t s) {
    const int tc = tile_width(g, kTileCorr);
    const size_t sm = (size_t)g.nz * tc * sizeof(double2);
    k_correction<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, sp, US, VS, WS, PHI, U, V, W, P, GP, tc);
    return cudaGetLastError();
}

cudaError_t launch_pcg_poisson(const GridDev& g, const Ops& ops, double2* PHI, double tol, cudaStream_t s) {
    const long long nsys = 2LL * (g.nm - 1);
    if (nsys <= 0) return cudaSuccess;
    k_pcg_poisson<<<(unsigned)((nsys + kPcgWarps - 1) / kPcgWarps), 32 * kPcgWarps, pcg_smem(g), s>>>(g, ops, PHI,
                                                                                                       tol);
    return cudaGetLastError();
}

cudaError_t launch_pcg_helmholtz(const GridDev& g, const Ops& ops, const StepParams& sp, Fields Out, double tol,
                                 cudaStream_t s) {
    const long long nsys = 6LL * g.nm;
    k_pcg_helmholtz<<<(unsigned)((nsys + kPcgWarps - 1) / kPcgWarps), 32 * kPcgWarps, pcg_smem(g), s>>>(
        g, ops, sp, Out, tol);
    return cudaGetLastError();
}

template <typename SrcC>
cudaError_t launch_rk_stage(const GridDev& g, const StepParams& sp, double coef, Fields F, FieldsT<SrcC> Src,
                            Fields Out, cudaStream_t s) {
    const size_t n = 3 * (size_t)g.nz * g.nm;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_rk_stage<SrcC><<<blocks, 256, 0, s>>>(g, sp, coef, F, Src, Out);
    return cudaGetLastError();
}
template cudaError_t launch_rk_stage<double2>(const GridDev&, const StepParams&, double, Fields, Fields, Fields,
                                              cudaStream_t);
template cudaError_t launch_rk_stage<float2>(const GridDev&, const StepParams&, double, Fields, FFields, Fields,
                                             cudaStream_t);

cudaError_t launch_apply_bc(const GridDev& g, double2* U, double2* V, double2* W, cudaStream_t s) {
    k_apply_bc<<<(2 * g.nm + 255) / 256, 256, 0, s>>>(g, U, V, W);
    return cudaGetLastError();
}

cudaError_t launch_divergence(const GridDev& g, const Ops& ops, const double2* U, const double2* V,
                              const double2* W, double2* DIV, cudaStream_t s) {
    const int tc = tile_width(g, kTileDiv);
    const size_t sm = (size_t)g.nz * tc * sizeof(double2);
    k_divergence<<<(g.nm + tc - 1) / tc, 256, sm, s>>>(g, ops, U, V, W, DIV, tc);
    return cudaGetLastError();
}

cudaError_t launch_grad_walls(const GridDev& g, const Ops& ops, const double2* P, double2* GP,
                              cudaStream_t s) {
    k_grad_walls<<<(g.nm + 255) / 256, 256, 0, s>>>(g, ops, P, GP);
    return cudaGetLastError();
}

cudaError_t launch_diag_reduce(const GridDev& g, const Ops& ops, const double* u, const double* v,
                               const double* w, double* partial, int nblocks, double* out,
                               cudaStream_t s) {
    // blocks per plane: nz of them fit the nblocks partial slots
    const int bx = std::max(1, std::min(nblocks / g.nz, (g.nx * g.ny + 255) / 256));
    if (bx * g.nz > nblocks) return cudaErrorInvalidValue;
    k_diag_partial<<<dim3(bx, g.nz), 256, 0, s>>>(g, ops.zw, u, v, w, partial);
    k_diag_final<<<1, 32, 0, s>>>(partial, bx * g.nz, out);
    return cudaGetLastError();
}

cudaError_t launch_diag_gather(const GridDev& g, const double2* U, const double2* V, const double2* W,
                               const dns3d_pi_state* pi, double* out, cudaStream_t s) {
    k_diag_gather<<<1, 128, 0, s>>>(g, U, V, W, pi, out);
    return cudaGetLastError();
}

cudaError_t launch_maxabs(const GridDev& g, const double* f, size_t n, double* partial, int nblocks,
                          double* out, cudaStream_t s) {
    (void)g;
    k_maxabs_partial<<<nblocks, 256, 0, s>>>(f, n, partial);
    k_max_final<<<1, 32, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}

cudaError_t launch_nonfinite_check(const double2* f, size_t n, int* flag, cudaStream_t s) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_nonfinite<<<blocks, 256, 0, s>>>(f, n, flag);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ ragged stages
// The non-transform stages of one run's step as k_stage bodies (ragged.cuh):
// virtual block b of a run is block b of the run's own launch of the same
// kernel, with the PI update as one extra block in front of the vorticity
// tiles.
namespace {

template <typename P, int N>
__device__ __forceinline__ FieldsT<P> desc_fields(void* const* p) {
    FieldsT<P> f;
#pragma unroll
    for (int i = 0; i < kMaxFields; ++i) f.p[i] = i < N ? static_cast<P*>(p[i]) : nullptr;
    return f;
}

__device__ __forceinline__ Fields fields3(double2* a, double2* b, double2* c) {
    Fields f;
#pragma unroll
    for (int i = 0; i < kMaxFields; ++i) f.p[i] = nullptr;
    f.p[0] = a;
    f.p[1] = b;
    f.p[2] = c;
    return f;
}

struct RsVort64 {
    static constexpr int kMinCtas = 2;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        if (b == 0) {
            pi_update_body(d.g, d.ops.zw, d.pp, d.U, d.pi, 0);
            return;
        }
        vorticity_body(d.g, d.ops, d.U, d.V, d.W, d.US, d.VS, d.WS, d.g.tc[kTileVort], b - 1);
    }
};

// the same with D1.u, D1.v on the tensor cores (runs with RunDesc::tcmask bit 1)
struct RsVort64Tc {
    static constexpr int kMinCtas = 1;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        if (b == 0) {
            pi_update_body(d.g, d.ops.zw, d.pp, d.U, d.pi, 0);
            return;
        }
        const int ntiles = (d.g.nm + kTcVortModes - 1) / kTcVortModes, chunk = d.vort_chunk;
        const int t0 = (b - 1) * chunk;
        const VortTcOp op{d.U, d.V, d.W, d.US, d.VS, d.WS};
        dz_tc_body(d.g, d.ops, op, t0, min(t0 + chunk, ntiles), d.tcerr);
    }
};

struct RsVort32 {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        if (b == 0) {
            pi_update_body(d.g, d.ops.zw, d.pp, d.U, d.pi, 0);
            return;
        }
        vorticity_mixed_body(d.g, d.mx, d.ops, d.U, d.V, d.W, desc_fields<float2, 6>(d.spec), d.g.tc[kTileVortM],
                             b - 1);
    }
};

template <typename T>
struct RsProd {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        const size_t n = (size_t)d.g.nx * d.g.ny * d.g.nz;
        if constexpr (sizeof(T) == 8)
            products_body(desc_fields<double, 6>(d.phys), desc_fields<double, 3>(d.phys), n, b, d.gx[kRsProd]);
        else
            products32_body(desc_fields<float, 6>(d.phys), desc_fields<float, 3>(d.phys), n, b, d.gx[kRsProd]);
    }
};

struct RsVisc64 {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        viscous_body<double2>(d.g, d.ops, d.sp, fields3(d.U, d.V, d.W), desc_fields<double2, 3>(d.src), d.GP, d.pi,
                              fields3(d.US, d.VS, d.WS), d.g.tc[kTileVisc], b);
    }
};

// the Crank-Nicolson solve on the tensor cores (runs with ops.tcA set)
struct RsVisc64Tc {
    static constexpr int kMinCtas = 2;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        // the phased schedule at every nz (one body per stage kernel)
        viscous_tc_body<false>(d.g, d.ops, d.sp, fields3(d.U, d.V, d.W), desc_fields<double2, 3>(d.src), d.GP, d.pi,
                               fields3(d.US, d.VS, d.WS), d.gx[kRsVisc], b, d.tcerr);
    }
};

struct RsVisc32 {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        viscous_mixed_body(d.g, d.mx, d.ops, d.sp, fields3(d.U, d.V, d.W), desc_fields<float2, 3>(d.src), d.GP,
                           fields3(d.US, d.VS, d.WS), d.g.tc[kTileViscM], b);
    }
};

struct RsViscMean {
    static constexpr int kMinCtas = 1;
    static __device__ __forceinline__ void run(const RunDesc& d, int) {
        viscous_body<float2>(d.g, d.ops, d.sp, fields3(d.U, d.V, d.W), desc_fields<float2, 3>(d.src), d.GP, d.pi,
                             fields3(d.US, d.VS, d.WS), 1, 0);
    }
};

struct RsPres64 {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        pressure_body(d.g, d.ops, d.sp, d.US, d.VS, d.WS, d.PHI, d.g.tc[kTilePres], b);
    }
};

// the Poisson solve of a right-hand side RsPresRhs left in PHI
struct RsPres64Tc {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        pressure_solve_body(d.g, d.ops, d.PHI, b);
    }
};

// the divergence right-hand side with D1.w* on the tensor cores (RunDesc::tcmask bit 4)
struct RsPresRhs64 {
    static constexpr int kMinCtas = 1;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        const int ntiles = (d.g.nm + kTcCorrModes - 1) / kTcCorrModes, chunk = d.corr_chunk;
        const int t0 = b * chunk;
        const PresRhsTcOp op{d.sp, d.US, d.VS, d.WS, d.PHI};
        dz_tc_body(d.g, d.ops, op, t0, min(t0 + chunk, ntiles), d.tcerr);
    }
};

struct RsPres32 {
    static constexpr int kMinCtas = 3;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        // runs with the Poisson refinement are not ragged-eligible (capi.cu)
        pressure_mixed_body<false>(d.g, d.mx, d.ops, d.sp, d.US, d.VS, d.WS, d.PHI, d.PHIZ, d.g.tc[kTilePresM], b);
    }
};

struct RsPresMean {
    static constexpr int kMinCtas = 1;
    static __device__ __forceinline__ void run(const RunDesc& d, int) {
        pressure_body(d.g, d.ops, d.sp, d.US, d.VS, d.WS, d.PHI, 1, 0);
        __syncthreads();  // phi of mode (0,0) written by this CTA
        dz_mean_mode_body(d.g, d.ops, d.PHI, d.PHIZ, 0);
    }
};

struct RsCorr64 {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        correction_body(d.g, d.ops, d.sp, d.US, d.VS, d.WS, d.PHI, d.U, d.V, d.W, d.P, d.GP, d.g.tc[kTileCorr], b);
    }
};

// the projection with D1.phi on the tensor cores (runs with RunDesc::tcmask bit 2)
struct RsCorr64Tc {
    static constexpr int kMinCtas = 1;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        const int ntiles = (d.g.nm + kTcCorrModes - 1) / kTcCorrModes, chunk = d.corr_chunk;
        const int t0 = b * chunk;
        const CorrTcOp op{d.sp, d.US, d.VS, d.WS, d.PHI, d.U, d.V, d.W, d.P, d.GP};
        dz_tc_body(d.g, d.ops, op, t0, min(t0 + chunk, ntiles), d.tcerr);
    }
};

struct RsCorr32 {
    static constexpr int kMinCtas = 4;
    static __device__ __forceinline__ void run(const RunDesc& d, int b) {
        correction_mixed_body(d.g, d.ops, d.sp, d.US, d.VS, d.WS, d.PHI, d.PHIZ, d.U, d.V, d.W, d.P, d.GP, b,
                              d.gx[kRsCorr]);
    }
};

}  // namespace

StageKernel ragged_kernel(int stage, bool mixed, int variant) {
    switch (stage) {
        case kRsVort:
            return mixed ? k_stage<RsVort32> : ((variant & kRvVortTc) ? k_stage<RsVort64Tc> : k_stage<RsVort64>);
        case kRsProd: return mixed ? k_stage<RsProd<float>> : k_stage<RsProd<double>>;
        case kRsVisc:
            return mixed ? k_stage<RsVisc32> : ((variant & kRvViscTc) ? k_stage<RsVisc64Tc> : k_stage<RsVisc64>);
        case kRsPres:
            return mixed ? k_stage<RsPres32> : ((variant & kRvPresTc) ? k_stage<RsPres64Tc> : k_stage<RsPres64>);
        case kRsPresRhs: return k_stage<RsPresRhs64>;
        case kRsCorr:
            return mixed ? k_stage<RsCorr32> : ((variant & kRvCorrTc) ? k_stage<RsCorr64Tc> : k_stage<RsCorr64>);
        case kRsViscMean: return k_stage<RsViscMean>;
        case kRsPresMean: return k_stage<RsPresMean>;
        case kRsFftYInv:
        case kRsFftC2R:
        case kRsFftR2C:
        case kRsFftYFwd: return ragged_fft_kernel(stage, mixed, (variant & kRvFftFx) != 0);
    }
    return nullptr;
}

int ragged_variant(const RunDesc& d) {
    return ((d.tcmask & 1) ? kRvVortTc : 0) | ((d.tcmask & 2) ? kRvCorrTc : 0) |
           ((d.tcmask & 4) && !d.sp.weak_form ? kRvPresTc : 0) |
           ((d.ops.tcA && d.sp.cn_identity) ? kRvViscTc : 0) | (d.fftfx ? kRvFftFx : 0);
}

void ragged_geometry(RunDesc& d) {
    const GridDev& g = d.g;
    auto cdiv = [](long long a, long long b) { return (int)((a + b - 1) / b); };
    for (int s = 0; s < kRsStages; ++s) d.gx[s] = 1;
    const int cy = fft_ct_per_cta(g.ny), rx = fft_ct_per_cta(g.nxh);
    d.gx[kRsFftYInv] = cdiv((long long)g.nz * g.nxhp, cy);
    d.gx[kRsFftC2R] = cdiv((long long)g.nz * g.ny, rx);
    d.gx[kRsProd] = cdiv((long long)g.nx * g.ny * g.nz, 4 * kStageThreads);
    d.gx[kRsFftR2C] = d.gx[kRsFftC2R];
    d.gx[kRsFftYFwd] = cdiv((long long)g.nz * d.ncol, cy);
    d.gx[kRsCorr] = cdiv((long long)g.nz * g.nm, 4 * kStageThreads);
    d.gx[kRsVisc] = tc_q_per_cta(d.ops.nq);  // operator indices per CTA of the tensor-core viscous body
    d.vort_chunk = tc_dz_chunk(g.nm, kTcVortModes);  // tiles per CTA of the tensor-core z-derivative bodies
    d.corr_chunk = tc_dz_chunk(g.nm, kTcCorrModes);
}

int ragged_tile_kernel(int stage, bool mixed) {
    switch (stage) {
        case kRsVort: return mixed ? kTileVortM : kTileVort;
        case kRsVisc: return mixed ? kTileViscM : kTileVisc;
        case kRsPres: return mixed ? kTilePresM : kTilePres;
        case kRsCorr: return mixed ? -1 : kTileCorr;
    }
    return -1;
}

int ragged_blocks(int stage, bool mixed, const RunDesc& d) {
    const GridDev& g = d.g;
    const int k = ragged_tile_kernel(stage, mixed);
    const int tiles = k >= 0 ? (g.nm + g.tc[k] - 1) / g.tc[k] : 0;
    switch (stage) {
        case kRsVort:
            if (!mixed && (ragged_variant(d) & kRvVortTc))
                return 1 + ((g.nm + kTcVortModes - 1) / kTcVortModes + d.vort_chunk - 1) / d.vort_chunk;
            return 1 + tiles;
        case kRsFftYInv:
        case kRsFftC2R: return 6 * d.gx[stage];
        case kRsFftR2C:
        case kRsFftYFwd: return 3 * d.gx[stage];
        case kRsProd: return d.gx[stage];
        case kRsVisc:
            if (!mixed && (ragged_variant(d) & kRvViscTc)) return (d.ops.nq + d.gx[kRsVisc] - 1) / d.gx[kRsVisc];
            return tiles;
        case kRsPres:
            if (!mixed && (ragged_variant(d) & kRvPresTc)) return (g.nm + fx_solve_modes(g.nz) - 1) / fx_solve_modes(g.nz);
            return tiles;
        case kRsPresRhs:
            if (!mixed && (ragged_variant(d) & kRvPresTc))
                return ((g.nm + kTcCorrModes - 1) / kTcCorrModes + d.corr_chunk - 1) / d.corr_chunk;
            return 0;
        case kRsCorr:
            if (!mixed && (ragged_variant(d) & kRvCorrTc))
                return ((g.nm + kTcCorrModes - 1) / kTcCorrModes + d.corr_chunk - 1) / d.corr_chunk;
            return mixed ? d.gx[stage] : tiles;
        case kRsViscMean:
        case kRsPresMean: return mixed ? 1 : 0;
    }
    return 0;
}

size_t ragged_smem(int stage, bool mixed, const RunDesc& d) {
    const GridDev& g = d.g;
    const size_t nz = g.nz;
    const int k = ragged_tile_kernel(stage, mixed);
    const int tc = k >= 0 ? g.tc[k] : 0;
    switch (stage) {
        case kRsVort:
            if (!mixed && (ragged_variant(d) & kRvVortTc)) return vorticity_tc_smem(g);
            return 2 * nz * tc * (mixed ? sizeof(float2) : sizeof(double2));
        case kRsVisc:
            if (!mixed && (ragged_variant(d) & kRvViscTc)) return viscous_tc_smem_nz<false>(g.nz);
            return mixed ? viscous_mixed_smem(g, tc) : 6 * nz * tc * sizeof(double2);
        case kRsPres:
            if (mixed) return pressure_mixed_smem(g, tc);
            return (ragged_variant(d) & kRvPresTc) ? fx_solve_smem(g.nz) : (2 * nz * tc + nz) * sizeof(double2);
        case kRsPresRhs: return (!mixed && (ragged_variant(d) & kRvPresTc)) ? vorticity_tc_smem(g) : 0;
        case kRsCorr:
            if (!mixed && (ragged_variant(d) & kRvCorrTc)) return vorticity_tc_smem(g);
            return mixed ? 0 : nz * tc * sizeof(double2);
        case kRsViscMean: return mixed ? 6 * nz * sizeof(double2) : 0;
        case kRsPresMean: return mixed ? 3 * nz * sizeof(double2) : 0;
    }
    return 0;
}

}  // namespace dns3d

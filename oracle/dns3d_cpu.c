/*
 * dns3d_cpu.c -- C/OpenMP restatement of the reference's 3D channel-flow time
 * step (TEST INFRASTRUCTURE AND CPU BASELINE ONLY).
 *
 * Only the test suite and the CPU legs of bench.py (`cpu_baseline` and
 * `--impl reference`) load this library, as a checker or as the timed CPU
 * baseline; the product library never calls it.
 *
 * It follows DNS_pressure_BC_3D.f90 (chandc/F90_DNS) as written, in physical
 * space, subroutine by subroutine, as the numpy restatement in dns3d_ref.py
 * does: every x/y derivative is an r2c -> multiply -> c2r round trip per
 * z-plane (compute_derivatives_3d, 3D:2321-2407), z-derivatives are d1 column
 * products, and the Helmholtz and Poisson matrices are rebuilt and LU-factored
 * with partial pivoting for every mode at every call, as the reference's zgesv
 * calls do (3D:1464-1505, 1680-1714).  Only the loops are parallel (OpenMP
 * over z-planes for the transforms and over modes for the solves).
 *
 * Third-party arithmetic restated:
 *  - FFTW3's 2D r2c / c2r (fftw3_dns_module.f90:72-130): a mixed-radix
 *    (4, 2, 3) Stockham complex FFT; the real x-transforms pack a length-nx
 *    real row into a length-nx/2 complex sequence.  c2r ignores the
 *    imaginary parts of the kx = 0 and kx = nx/2 inputs (FFTW's semantics for
 *    non-Hermitian input) and the wrapper divides by nx*ny.
 *  - LAPACK zgesv: LU with partial pivoting.  The matrices are real (complex
 *    storage with zero imaginary part), so the pivot search on |a| and the
 *    elimination are done in real arithmetic and applied to the complex
 *    right-hand side.
 *
 * Layout: u(nx,ny,nz) Fortran order == C u[k][j][i]; spectra [k][j][kx],
 * kx = 0..nx/2.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nx, ny, nz, istart;
    int use_crank_nicolson, flow_control_method, controller_update_freq;
    int enable_perturbations, use_analytical_perturbations, analytical_mode_x, analytical_mode_y;
    int use_weak_form_divergence, use_dealias_23_rule, lgl_dmatrix_guard;
    double dt, re, xlen, ylen, u_centerline;
    double target_pressure_gradient, target_bulk_velocity, controller_gain, perturbation_amplitude;
} cpu_config;

typedef struct { double re, im; } cx;

static inline cx cmul(cx a, cx b) { cx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cx cadd(cx a, cx b) { cx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cx csub(cx a, cx b) { cx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cx cconj(cx a) { cx r = {a.re, -a.im}; return r; }

/* ------------------------------------------------------------------ FFT */
typedef struct {
    int n, nf, f[40];
    cx* w; /* w[t] = exp(-2 pi i t / n) */
} plan1d;

static int plan_init(plan1d* p, int n) {
    p->n = n;
    p->nf = 0;
    int m = n;
    while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
    while (m % 3 == 0) { p->f[p->nf++] = 3; m /= 3; }
    if (m != 1) return -1;
    p->w = (cx*)malloc(sizeof(cx) * (size_t)(n > 0 ? n : 1));
    if (!p->w) return -1;
    const double pi = 3.14159265358979323846;
    for (int t = 0; t < n; ++t) {
        p->w[t].re = cos(2.0 * pi * t / n);
        p->w[t].im = -sin(2.0 * pi * t / n);
    }
    return 0;
}

static void plan_free(plan1d* p) { free(p->w); p->w = NULL; }

/* Unnormalised DFT of length n, sign -1 (forward) or +1 (inverse), in place
 * in x with scratch y (both length n).  Stockham autosort, decimation in
 * time: a pass of radix r over l finished sub-transforms reads X[j][k'+q m]
 * (stored at j*r*m + k' + q*m), twiddles by w^(j q m) and writes the r
 * outputs to (j + l q')*m + k'. */
static void fft1d(const plan1d* p, cx* x, cx* y, int sign) {
    const int n = p->n;
    int l = 1;
    cx* src = x;
    cx* dst = y;
    for (int s = 0; s < p->nf; ++s) {
        const int r = p->f[s];
        const int m = n / (l * r);
        for (int j = 0; j < l; ++j) {
            for (int k = 0; k < m; ++k) {
                cx a[4];
                for (int q = 0; q < r; ++q) {
                    cx v = src[j * r * m + k + q * m];
                    const int t = (int)(((long long)j * q * m) % n);
                    cx tw = p->w[t];
                    if (sign > 0) tw = cconj(tw);
                    a[q] = q ? cmul(v, tw) : v;
                }
                cx b[4];
                if (r == 2) {
                    b[0] = cadd(a[0], a[1]);
                    b[1] = csub(a[0], a[1]);
                } else if (r == 4) {
                    const cx s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
                    const cx s13 = cadd(a[1], a[3]), d13 = csub(a[1], a[3]);
                    /* -i*sign*d13 : forward multiplies by -i, inverse by +i */
                    cx rot;
                    if (sign < 0) { rot.re = d13.im; rot.im = -d13.re; }
                    else { rot.re = -d13.im; rot.im = d13.re; }
                    b[0] = cadd(s02, s13);
                    b[1] = cadd(d02, rot);
                    b[2] = csub(s02, s13);
                    b[3] = csub(d02, rot);
                } else { /* r == 3 */
                    const double c3 = -0.5, s3 = (sign < 0 ? -1.0 : 1.0) * 0.86602540378443864676;
                    const cx t1 = cadd(a[1], a[2]);
                    const cx t2 = csub(a[1], a[2]);
                    const cx m1 = {a[0].re + c3 * t1.re, a[0].im + c3 * t1.im};
                    const cx m2 = {-s3 * t2.im, s3 * t2.re}; /* i*s3*t2 */
                    b[0] = cadd(a[0], t1);
                    b[1] = cadd(m1, m2);
                    b[2] = csub(m1, m2);
                }
                for (int q = 0; q < r; ++q) dst[(j + l * q) * m + k] = b[q];
            }
        }
        l *= r;
        cx* t = src;
        src = dst;
        dst = t;
    }
    if (src != x) memcpy(x, src, sizeof(cx) * (size_t)n);
}

typedef struct {
    int nx, ny, nxh, nxhp;
    plan1d px; /* length nx/2 (packed real rows) */
    plan1d py; /* length ny */
    cx* wr;    /* exp(-2 pi i k / nx), k = 0..nx/2 */
} plan2d;

static int plan2d_init(plan2d* p, int nx, int ny) {
    p->nx = nx;
    p->ny = ny;
    p->nxh = nx / 2;
    p->nxhp = nx / 2 + 1;
    if (plan_init(&p->px, p->nxh) || plan_init(&p->py, ny)) return -1;
    p->wr = (cx*)malloc(sizeof(cx) * (size_t)p->nxhp);
    const double pi = 3.14159265358979323846;
    for (int k = 0; k <= p->nxh; ++k) {
        p->wr[k].re = cos(2.0 * pi * k / nx);
        p->wr[k].im = -sin(2.0 * pi * k / nx);
    }
    return 0;
}

static void plan2d_free(plan2d* p) {
    plan_free(&p->px);
    plan_free(&p->py);
    free(p->wr);
}

/* per-thread scratch: 3 * max(nx, ny) complex */
static void r2c_plane(const plan2d* p, const double* in, cx* out, cx* s) {
    const int nx = p->nx, ny = p->ny, N = p->nxh, nxhp = p->nxhp;
    cx* z = s;
    cx* y = s + (nx > ny ? nx : ny);
    for (int j = 0; j < ny; ++j) {
        const double* row = in + (size_t)j * nx;
        for (int n = 0; n < N; ++n) { z[n].re = row[2 * n]; z[n].im = row[2 * n + 1]; }
        fft1d(&p->px, z, y, -1);
        cx* o = out + (size_t)j * nxhp;
        for (int k = 0; k <= N; ++k) {
            const cx zk = z[k % N];
            const cx zc = cconj(z[(N - k) % N]);
            const cx e = {0.5 * (zk.re + zc.re), 0.5 * (zk.im + zc.im)};
            const cx d = csub(zk, zc);
            const cx od = {0.5 * d.im, -0.5 * d.re}; /* (zk - zc) / (2i) */
            o[k] = cadd(e, cmul(p->wr[k], od));
        }
    }
    cx* col = s;
    for (int kx = 0; kx < nxhp; ++kx) {
        for (int j = 0; j < ny; ++j) col[j] = out[(size_t)j * nxhp + kx];
        fft1d(&p->py, col, y, -1);
        for (int j = 0; j < ny; ++j) out[(size_t)j * nxhp + kx] = col[j];
    }
}

/* c2r of `in` (destroyed) into `out`, divided by nx*ny */
static void c2r_plane(const plan2d* p, cx* in, double* out, cx* s) {
    const int nx = p->nx, ny = p->ny, N = p->nxh, nxhp = p->nxhp;
    cx* col = s;
    cx* y = s + (nx > ny ? nx : ny);
    for (int kx = 0; kx < nxhp; ++kx) {
        for (int j = 0; j < ny; ++j) col[j] = in[(size_t)j * nxhp + kx];
        fft1d(&p->py, col, y, +1);
        for (int j = 0; j < ny; ++j) in[(size_t)j * nxhp + kx] = col[j];
    }
    const double sc = 1.0 / ((double)nx * (double)ny);
    cx* z = s;
    for (int j = 0; j < ny; ++j) {
        cx* X = in + (size_t)j * nxhp;
        X[0].im = 0.0; /* the 1D c2r reads only the real parts of the ends */
        X[N].im = 0.0;
        for (int k = 0; k < N; ++k) {
            const cx xk = X[k], xc = cconj(X[N - k]);
            const cx e = cadd(xk, xc);
            const cx o = cmul(csub(xk, xc), cconj(p->wr[k]));
            z[k].re = e.re - o.im; /* e + i o */
            z[k].im = e.im + o.re;
        }
        fft1d(&p->px, z, y, +1);
        double* row = out + (size_t)j * nx;
        for (int n = 0; n < N; ++n) { row[2 * n] = z[n].re * sc; row[2 * n + 1] = z[n].im * sc; }
    }
}

/* ------------------------------------------------------------------ LGL */
static void legendre_d(int n, double x, double* p, double* dp, double* d2p) {
    if (n == 0) { *p = 1.0; *dp = 0.0; *d2p = 0.0; return; }
    if (n == 1) { *p = x; *dp = 1.0; *d2p = 0.0; return; }
    double p0 = 1.0, dp0 = 0.0, d2p0 = 0.0, p1 = x, dp1 = 1.0, d2p1 = 0.0;
    for (int k = 2; k <= n; ++k) {
        const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        const double dp2 = ((2 * k - 1) * (x * dp1 + p1) - (k - 1) * dp0) / k;
        const double d2p2 = ((2 * k - 1) * (x * d2p1 + 2.0 * dp1) - (k - 1) * d2p0) / k;
        p0 = p1; p1 = p2; dp0 = dp1; dp1 = dp2; d2p0 = d2p1; d2p1 = d2p2;
    }
    *p = p1; *dp = dp1; *d2p = d2p1;
}

/* lgl_nodes_weights, lgl_module.f90:30-80 */
static void lgl(int n, double* x, double* w) {
    const double pi_l = 3.14159265358979323846;
    x[0] = -1.0; x[n - 1] = 1.0;
    w[0] = w[n - 1] = 2.0 / (double)(n * (n - 1));
    for (int i = 2; i < n; ++i) {
        double xi = -cos(pi_l * (i - 1) / (n - 1));
        for (int it = 0; it < 100; ++it) {
            double p, dp, d2p;
            const double xo = xi;
            legendre_d(n - 1, xi, &p, &dp, &d2p);
            xi = xo - dp / d2p;
            if (fabs(xi - xo) < 1.0e-15) break;
        }
        x[i - 1] = xi;
        double p, dp, d2p;
        legendre_d(n - 1, xi, &p, &dp, &d2p);
        w[i - 1] = 2.0 / ((double)(n * (n - 1)) * p * p);
    }
}

/* differentiation_matrix, lgl_module.f90:211-263 (row-major d[i*n+j]) */
static void dmatrix(int n, const double* x, int guard, double* d) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            if (i == j) {
                double s = 0.0;
                for (int k = 0; k < n; ++k)
                    if (k != i) s += 1.0 / (x[i] - x[k]);
                d[i * n + i] = s;
            } else {
                double p1 = 1.0, p2 = 1.0;
                for (int k = 0; k < n; ++k) {
                    if (k != i && k != j) p1 *= x[i] - x[k];
                    if (k != j) p2 *= x[j] - x[k];
                }
                d[i * n + j] = (fabs(p2) > 1.0e-15 || !guard) ? p1 / p2 : 0.0;
            }
        }
}

/* ------------------------------------------------------------------ state */
typedef struct {
    cpu_config c;
    int nthreads;
    int nx, ny, nz, nxhp;
    size_t pl, spl, N, NS; /* plane / spectral plane / field sizes */
    plan2d fp;
    double *zpts, *zwts, *d1, *d2, *xw, *yw;
    double alpha, beta, ybar;
    double *u, *v, *w, *p, *gpx, *gpy, *gpz;
    double *t[24]; /* physical work fields */
    cx *sa, *sb;   /* spectral work fields */
    cx* scratch;   /* per thread */
    size_t scr;
    /* PI globals (3D:75-89) */
    double current_pressure_gradient, current_bulk_velocity, bulk_velocity_error;
    double bulk_velocity_error_integral, bulk_velocity_error_prev, pressure_gradient_sum, avg_pressure_gradient;
    int pressure_gradient_count;
    int istep;
    double time;
} cpu_run;

static cx* thread_scratch(cpu_run* r) {
#ifdef _OPENMP
    return r->scratch + (size_t)omp_get_thread_num() * r->scr;
#else
    return r->scratch;
#endif
}

static void r2c_field(cpu_run* r, const double* f, cx* F) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(r->nthreads)
    for (int k = 0; k < r->nz; ++k) r2c_plane(&r->fp, f + k * r->pl, F + k * r->spl, thread_scratch(r));
}

static void c2r_field(cpu_run* r, cx* F, double* f) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(r->nthreads)
    for (int k = 0; k < r->nz; ++k) c2r_plane(&r->fp, F + k * r->spl, f + k * r->pl, thread_scratch(r));
}

/* dfdz(i,j,:) = (2/ybar) matmul(d1, f(i,j,:)) (3D:2351-2357) */
static void ddz(cpu_run* r, const double* f, double* out) {
    const int nz = r->nz;
    const size_t pl = r->pl;
    const double zs = 2.0 / r->ybar;
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
    for (int j = 0; j < r->ny; ++j) {
        for (int k = 0; k < nz; ++k) {
            double* o = out + k * pl + (size_t)j * r->nx;
            for (int i = 0; i < r->nx; ++i) o[i] = 0.0;
            for (int m = 0; m < nz; ++m) {
                const double dk = r->d1[k * nz + m];
                const double* fm = f + m * pl + (size_t)j * r->nx;
                for (int i = 0; i < r->nx; ++i) o[i] += dk * fm[i];
            }
            for (int i = 0; i < r->nx; ++i) o[i] *= zs;
        }
    }
}

/* compute_derivatives_3d (3D:2321-2407): dx, dy by r2c * (0, xw|yw) c2r per
 * plane, dz by d1; any output may be NULL */
static void derivatives(cpu_run* r, const double* f, double* fx, double* fy, double* fz) {
    if (fz) ddz(r, f, fz);
    if (!fx && !fy) return;
    const int nz = r->nz, ny = r->ny, nxhp = r->nxhp;
#pragma omp parallel for schedule(dynamic, 1) num_threads(r->nthreads)
    for (int k = 0; k < nz; ++k) {
        cx* s = thread_scratch(r);
        cx* F = r->sa + k * r->spl;
        cx* G = r->sb + k * r->spl;
        r2c_plane(&r->fp, f + k * r->pl, F, s);
        if (fx) {
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nxhp; ++i) {
                    const cx a = F[(size_t)j * nxhp + i];
                    const cx m = {0.0, r->xw[i]};
                    G[(size_t)j * nxhp + i] = cmul(a, m);
                }
            c2r_plane(&r->fp, G, fx + k * r->pl, s);
        }
        if (fy) {
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nxhp; ++i) {
                    const cx a = F[(size_t)j * nxhp + i];
                    const cx m = {0.0, r->yw[j]};
                    G[(size_t)j * nxhp + i] = cmul(a, m);
                }
            c2r_plane(&r->fp, G, fy + k * r->pl, s);
        }
    }
}

/* compute_laplacian_3d (3D:1564-1606): (2/ybar)^2 d2 f^ - (xsq+ysq) f^ */
static void laplacian(cpu_run* r, const double* f, double* out) {
    const int nz = r->nz, ny = r->ny, nxhp = r->nxhp;
    r2c_field(r, f, r->sa);
    const double zs2 = (2.0 / r->ybar) * (2.0 / r->ybar);
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
            cx* o = r->sb + k * r->spl + (size_t)j * nxhp;
            for (int i = 0; i < nxhp; ++i) {
                cx acc = {0.0, 0.0};
                for (int m = 0; m < nz; ++m) {
                    const cx a = r->sa[m * r->spl + (size_t)j * nxhp + i];
                    acc.re += r->d2[k * nz + m] * a.re;
                    acc.im += r->d2[k * nz + m] * a.im;
                }
                const cx a = r->sa[k * r->spl + (size_t)j * nxhp + i];
                const double ks = r->xw[i] * r->xw[i] + r->yw[j] * r->yw[j];
                o[i].re = acc.re * zs2 - ks * a.re;
                o[i].im = acc.im * zs2 - ks * a.im;
            }
        }
    c2r_field(r, r->sb, out);
}

/* LU with partial pivoting of a real n x n matrix (row-major, in place) and
 * solve for one complex right-hand side (zgesv on a real-valued matrix) */
static int lu_solve(int n, double* a, cx* b) {
    for (int c = 0; c < n; ++c) {
        int piv = c;
        double best = fabs(a[c * n + c]);
        for (int i = c + 1; i < n; ++i)
            if (fabs(a[i * n + c]) > best) { best = fabs(a[i * n + c]); piv = i; }
        if (best == 0.0) return -1;
        if (piv != c) {
            for (int j = 0; j < n; ++j) { const double t = a[c * n + j]; a[c * n + j] = a[piv * n + j]; a[piv * n + j] = t; }
            const cx t = b[c]; b[c] = b[piv]; b[piv] = t;
        }
        const double inv = 1.0 / a[c * n + c];
        for (int i = c + 1; i < n; ++i) {
            const double l = a[i * n + c] * inv;
            if (l == 0.0) continue;
            for (int j = c + 1; j < n; ++j) a[i * n + j] -= l * a[c * n + j];
            b[i].re -= l * b[c].re;
            b[i].im -= l * b[c].im;
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        cx s = b[i];
        for (int j = i + 1; j < n; ++j) { s.re -= a[i * n + j] * b[j].re; s.im -= a[i * n + j] * b[j].im; }
        b[i].re = s.re / a[i * n + i];
        b[i].im = s.im / a[i * n + i];
    }
    return 0;
}

/* S_kn = sum_m d1(m,k) d1(m,n) zwts(m) (2/ybar) (3D:1464-1472) */
static void stiffness(cpu_run* r, double* S) {
    const int nz = r->nz;
    for (int k = 0; k < nz; ++k)
        for (int n = 0; n < nz; ++n) {
            double s = 0.0;
            for (int m = 0; m < nz; ++m) s += r->d1[m * nz + k] * r->d1[m * nz + n] * r->zwts[m];
            S[k * nz + n] = s * (2.0 / r->ybar);
        }
}

/* solve_viscous_helmholtz (3D:1425-1521), lifting quirk included: interior
 * rows lose H(k,1) bc1 + H(k,nz) bc2, rows 1 and nz become identity rows with
 * columns 1 and nz kept (the wall data enters twice) */
static int helmholtz(cpu_run* r, const double* rhs, double theta, const double* bc1, const double* bc2, double* out) {
    const int nz = r->nz, ny = r->ny, nxhp = r->nxhp;
    const double f = theta * r->c.dt / r->c.re, half = r->ybar / 2.0;
    r2c_field(r, rhs, r->sa);
    cx* B1 = r->sb;  /* two spare planes of sb hold the wall spectra */
    cx* B2 = r->sb + r->spl;
    cx* s0 = thread_scratch(r);
    r2c_plane(&r->fp, bc1, B1, s0);
    r2c_plane(&r->fp, bc2, B2, s0);
    double* S = (double*)malloc(sizeof(double) * nz * nz);
    stiffness(r, S);
    int bad = 0;
#pragma omp parallel num_threads(r->nthreads) reduction(| : bad)
    {
        double* H = (double*)malloc(sizeof(double) * nz * nz);
        cx* b = (cx*)malloc(sizeof(cx) * nz);
#pragma omp for schedule(dynamic, 16)
        for (int m = 0; m < ny * nxhp; ++m) {
            const int j = m / nxhp, i = m - j * nxhp;
            const double ks = r->xw[i] * r->xw[i] + r->yw[j] * r->yw[j];
            for (int k = 0; k < nz; ++k)
                for (int n = 0; n < nz; ++n) H[k * nz + n] = f * S[k * nz + n];
            for (int k = 0; k < nz; ++k) H[k * nz + k] += (1.0 + f * ks) * r->zwts[k] * half;
            for (int k = 0; k < nz; ++k) {
                const cx a = r->sa[k * r->spl + m];
                b[k].re = a.re * r->zwts[k] * half;
                b[k].im = a.im * r->zwts[k] * half;
            }
            const cx c1 = B1[m], c2 = B2[m];
            for (int k = 1; k < nz - 1; ++k) {
                b[k].re -= H[k * nz] * c1.re + H[k * nz + nz - 1] * c2.re;
                b[k].im -= H[k * nz] * c1.im + H[k * nz + nz - 1] * c2.im;
            }
            b[0] = c1;
            b[nz - 1] = c2;
            for (int n = 0; n < nz; ++n) { H[n] = 0.0; H[(nz - 1) * nz + n] = 0.0; }
            H[0] = 1.0;
            H[(nz - 1) * nz + nz - 1] = 1.0;
            if (lu_solve(nz, H, b)) bad = 1;
            for (int k = 0; k < nz; ++k) r->sa[k * r->spl + m] = b[k];
        }
        free(H);
        free(b);
    }
    free(S);
    if (bad) return -1;
    c2r_field(r, r->sa, out);
    return 0;
}

/* calculate_bulk_velocity_3d (3D:2434-2464) */
static double bulk_velocity(cpu_run* r, const double* u) {
    double vol = 0.0, wsum = 0.0;
    for (int k = 0; k < r->nz; ++k) {
        double s = 0.0;
        const double* uk = u + k * r->pl;
        for (size_t i = 0; i < r->pl; ++i) s += uk[i];
        vol += s * r->zwts[k];
        wsum += r->zwts[k];
    }
    return vol / ((double)r->nx * (double)r->ny * wsum);
}

/* update_pressure_gradient_3d (3D:2488-2549) */
static void update_pressure_gradient(cpu_run* r, int istep) {
    const cpu_config* c = &r->c;
    if (istep % c->controller_update_freq != 0) return;
    r->current_bulk_velocity = bulk_velocity(r, r->u);
    r->bulk_velocity_error = c->target_bulk_velocity - r->current_bulk_velocity;
    const double kp = c->controller_gain, ki = 0.05 * c->controller_gain, base = 3.0 / c->re;
    const double un = base + kp * r->bulk_velocity_error + ki * r->bulk_velocity_error_integral;
    const double cl = un < 0.0 ? 0.0 : (un > 10.0 ? 10.0 : un);
    if (fabs(cl - un) < 1.0e-12) {
        if (istep <= c->controller_update_freq)
            r->bulk_velocity_error_integral += r->bulk_velocity_error * c->dt;
        else
            r->bulk_velocity_error_integral += 0.5 * c->dt * (r->bulk_velocity_error_prev + r->bulk_velocity_error);
    }
    r->bulk_velocity_error_prev = r->bulk_velocity_error;
    r->current_pressure_gradient = cl;
    r->pressure_gradient_sum += cl;
    r->pressure_gradient_count += 1;
    r->avg_pressure_gradient = r->pressure_gradient_sum / (double)r->pressure_gradient_count;
}

/* apply_dealias_truncation (3D:1163-1193) on a spectral field */
static void dealias(cpu_run* r, cx* F) {
    const int kxm = ((r->nx / 2) * 2) / 3, kym = ((r->ny / 2) * 2) / 3;
    for (int k = 0; k < r->nz; ++k)
        for (int j = 1; j <= r->ny; ++j)
            for (int i = 1; i <= r->nxhp; ++i) {
                int zero = (i - 1) > kxm;
                if (!zero) zero = (j <= r->ny / 2 + 1) ? (j - 1) > kym : abs(j - 1 - r->ny) > kym;
                if (zero) {
                    cx* a = &F[k * r->spl + (size_t)(j - 1) * r->nxhp + (i - 1)];
                    a->re = 0.0;
                    a->im = 0.0;
                }
            }
}

/* compute_source_terms_3d (3D:1032-1148) into t[0..2] */
static void source_terms(cpu_run* r) {
    double **T = r->t, *u = r->u, *v = r->v, *w = r->w;
    const size_t N = r->N;
    /* t3..t11: ux uy uz vx vy vz wx wy wz */
    derivatives(r, u, T[3], T[4], T[5]);
    derivatives(r, v, T[6], T[7], T[8]);
    derivatives(r, w, T[9], T[10], T[11]);
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
    for (size_t i = 0; i < N; ++i) {
        const double ox = T[10][i] - T[8][i]; /* wy - vz (3D:1077-1079) */
        const double oy = T[5][i] - T[9][i];  /* uz - wx */
        const double oz = T[6][i] - T[4][i];  /* vx - uy */
        T[0][i] = v[i] * oz - w[i] * oy;      /* 3D:1089-1091 */
        T[1][i] = w[i] * ox - u[i] * oz;
        T[2][i] = u[i] * oy - v[i] * ox;
    }
    if (r->c.use_dealias_23_rule)
        for (int f = 0; f < 3; ++f) {
            r2c_field(r, T[f], r->sa);
            dealias(r, r->sa);
            c2r_field(r, r->sa, T[f]);
        }
    if (r->c.flow_control_method == 1) r->current_pressure_gradient = r->c.target_pressure_gradient;
    else if (r->c.flow_control_method == 2) update_pressure_gradient(r, r->c.istart); /* 3D:1118 */
    const double g = r->current_pressure_gradient;
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
    for (size_t i = 0; i < N; ++i) T[0][i] += g;
}

/* viscous_step_3d (3D:1285-1332): t[0..2] sources -> t[12..14] u*, v*, w* */
static int viscous_step(cpu_run* r) {
    double** T = r->t;
    const double theta = r->c.use_crank_nicolson ? 0.5 : 1.0, dt = r->c.dt;
    const size_t N = r->N, pl = r->pl;
    double* vel[3] = {r->u, r->v, r->w};
    for (int f = 0; f < 3; ++f) {
        double* rhs = T[15 + f];
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
        for (size_t i = 0; i < N; ++i) rhs[i] = vel[f][i] + dt * T[f][i];
        if (theta < 1.0) {
            laplacian(r, vel[f], T[18]);
            const double fac = 0.5 * dt / r->c.re;
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
            for (size_t i = 0; i < N; ++i) rhs[i] += fac * T[18][i];
        }
    }
    double* b1 = T[19];
    double* b2 = T[19] + pl;
    for (int f = 0; f < 3; ++f) {
        const double* g = f == 0 ? r->gpx : (f == 1 ? r->gpy : NULL);
        for (size_t i = 0; i < pl; ++i) {
            b1[i] = g ? -dt * g[i] : 0.0;
            b2[i] = g ? -dt * g[(size_t)(r->nz - 1) * pl + i] : 0.0;
        }
        if (helmholtz(r, T[15 + f], theta, b1, b2, T[12 + f])) return -1;
    }
    return 0;
}

/* solve_pressure_3d (3D:1631-1835) -> phi in t[20] */
static int solve_pressure(cpu_run* r) {
    double** T = r->t;
    const int nz = r->nz, ny = r->ny, nxhp = r->nxhp;
    const double half = r->ybar / 2.0, dt = r->c.dt;
    if (!r->c.use_weak_form_divergence) {
        /* div = compute_divergence_3d(u*,v*,w*)/dt (3D:1670-1671) */
        derivatives(r, T[12], T[3], NULL, NULL);
        derivatives(r, T[13], NULL, T[4], NULL);
        derivatives(r, T[14], NULL, NULL, T[5]);
        const size_t N = r->N;
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
        for (size_t i = 0; i < N; ++i) T[21][i] = (T[3][i] + T[4][i] + T[5][i]) / dt;
        r2c_field(r, T[21], r->sa);
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
        for (int k = 0; k < nz; ++k)
            for (size_t m = 0; m < r->spl; ++m) {
                cx* a = &r->sa[k * r->spl + m];
                a->re *= 0.5 * r->ybar * r->zwts[k];
                a->im *= 0.5 * r->ybar * r->zwts[k];
            }
    } else {
        /* weak form (3D:1749-1835) */
        cx* U = r->sa;
        cx* V = r->sb;
        r2c_field(r, T[12], U);
        r2c_field(r, T[13], V);
        cx* Wh = (cx*)malloc(sizeof(cx) * r->NS);
        r2c_field(r, T[14], Wh);
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
        for (int m = 0; m < ny * nxhp; ++m) {
            const int j = m / nxhp, i = m - j * nxhp;
            for (int k = 0; k < nz; ++k) {
                const cx a = U[k * r->spl + m], b = V[k * r->spl + m];
                /* -(i xw u + i yw v) w_k ybar/2 */
                cx hz = {-(r->xw[i] * a.im + r->yw[j] * b.im), r->xw[i] * a.re + r->yw[j] * b.re};
                cx vert = {0.0, 0.0};
                for (int mm = 0; mm < nz; ++mm) {
                    const double c = r->d1[mm * nz + k] * r->zwts[mm];
                    vert.re += c * Wh[mm * r->spl + m].re;
                    vert.im += c * Wh[mm * r->spl + m].im;
                }
                vert.re *= 2.0 / r->ybar;
                vert.im *= 2.0 / r->ybar;
                U[k * r->spl + m].re = (-hz.re * r->zwts[k] * half - vert.re) / dt;
                U[k * r->spl + m].im = (-hz.im * r->zwts[k] * half - vert.im) / dt;
            }
        }
        free(Wh);
    }
    double* S = (double*)malloc(sizeof(double) * nz * nz);
    stiffness(r, S);
    int bad = 0;
#pragma omp parallel num_threads(r->nthreads) reduction(| : bad)
    {
        double* P = (double*)malloc(sizeof(double) * nz * nz);
        cx* b = (cx*)malloc(sizeof(cx) * nz);
#pragma omp for schedule(dynamic, 16)
        for (int m = 0; m < ny * nxhp; ++m) {
            const int j = m / nxhp, i = m - j * nxhp;
            const double ks = r->xw[i] * r->xw[i] + r->yw[j] * r->yw[j];
            for (int k = 0; k < nz; ++k)
                for (int n = 0; n < nz; ++n) P[k * nz + n] = -S[k * nz + n];
            for (int k = 0; k < nz; ++k) P[k * nz + k] -= ks * r->zwts[k] * half;  /* 3D:1684-1692 */
            for (int k = 0; k < nz; ++k) b[k] = r->sa[k * r->spl + m];
            if (m == 0) { /* mode (1,1) pin (3D:1702-1711) */
                for (int n = 0; n < nz; ++n) { P[n] = 0.0; P[n * nz] = 0.0; }
                P[0] = 1.0;
                b[0].re = b[0].im = 0.0;
            }
            if (lu_solve(nz, P, b)) bad = 1;
            for (int k = 0; k < nz; ++k) r->sa[k * r->spl + m] = b[k];
        }
        free(P);
        free(b);
    }
    free(S);
    if (bad) return -1;
    c2r_field(r, r->sa, T[20]);
    return 0;
}

/* pressure_correction_3d (3D:1903-1929) */
static void pressure_correction(cpu_run* r) {
    double** T = r->t;
    const size_t N = r->N;
    const double dt = r->c.dt;
    derivatives(r, T[20], T[3], T[4], T[5]);
#pragma omp parallel for schedule(static) num_threads(r->nthreads)
    for (size_t i = 0; i < N; ++i) {
        r->u[i] = T[12][i] - dt * T[3][i];
        r->v[i] = T[13][i] - dt * T[4][i];
        r->w[i] = T[14][i] - dt * T[5][i];
        r->p[i] += T[20][i];
    }
    derivatives(r, r->p, r->gpx, r->gpy, r->gpz);
}

/* apply_boundary_conditions_3d (3D:1953-1972) */
static void apply_bc(cpu_run* r) {
    const size_t pl = r->pl, top = (size_t)(r->nz - 1) * pl;
    for (size_t i = 0; i < pl; ++i) {
        r->u[i] = r->v[i] = r->w[i] = 0.0;
        r->u[top + i] = r->v[top + i] = r->w[top + i] = 0.0;
    }
}

/* ------------------------------------------------------------------ API */
void cpu_destroy(void* h);

void* cpu_create(const cpu_config* c, int nthreads) {
    if (!c || c->nx < 4 || c->ny < 2 || c->nz < 3 || (c->nx % 2)) return NULL;
    /* only the analytical initial perturbation is restated here; runs with
     * the random one are set up through cpu_set_state */
    if (c->enable_perturbations && !c->use_analytical_perturbations) return NULL;
    cpu_run* r = (cpu_run*)calloc(1, sizeof(cpu_run));
    if (!r) return NULL;
    r->c = *c;
#ifdef _OPENMP
    r->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    r->nthreads = 1;
    (void)nthreads;
#endif
    r->nx = c->nx; r->ny = c->ny; r->nz = c->nz; r->nxhp = c->nx / 2 + 1;
    r->pl = (size_t)c->nx * c->ny;
    r->spl = (size_t)r->nxhp * c->ny;
    r->N = r->pl * c->nz;
    r->NS = r->spl * c->nz;
    if (plan2d_init(&r->fp, c->nx, c->ny)) { cpu_destroy(r); return NULL; }
    const double pi = 4.0 * atan(1.0); /* 3D:43 */
    r->alpha = 2.0 * pi / c->xlen;       /* 3D:740-742 */
    r->beta = 2.0 * pi / c->ylen;
    r->ybar = 2.0;
    const int nz = c->nz;
    r->zpts = (double*)malloc(sizeof(double) * nz);
    r->zwts = (double*)malloc(sizeof(double) * nz);
    r->d1 = (double*)malloc(sizeof(double) * nz * nz);
    r->d2 = (double*)calloc((size_t)nz * nz, sizeof(double));
    r->xw = (double*)malloc(sizeof(double) * r->nxhp);
    r->yw = (double*)malloc(sizeof(double) * c->ny);
    lgl(nz, r->zpts, r->zwts);
    dmatrix(nz, r->zpts, c->lgl_dmatrix_guard, r->d1);
    for (int i = 0; i < nz; ++i)
        for (int j = 0; j < nz; ++j) {
            double s = 0.0;
            for (int k = 0; k < nz; ++k) s += r->d1[i * nz + k] * r->d1[k * nz + j];
            r->d2[i * nz + j] = s; /* d2 = d1 d1 (3D:801) */
        }
    for (int i = 0; i < r->nxhp; ++i) r->xw[i] = (double)i * r->alpha; /* 3D:780-783 */
    for (int j = 1; j <= c->ny; ++j)                                    /* 3D:789-796 */
        r->yw[j - 1] = (j <= c->ny / 2 + 1 ? (double)(j - 1) : (double)(j - 1 - c->ny)) * 2.0 * pi / c->ylen;
    double** fields[7] = {&r->u, &r->v, &r->w, &r->p, &r->gpx, &r->gpy, &r->gpz};
    for (int f = 0; f < 7; ++f) *fields[f] = (double*)calloc(r->N, sizeof(double));
    for (int f = 0; f < 24; ++f) r->t[f] = (double*)calloc(r->N, sizeof(double));
    r->sa = (cx*)calloc(r->NS, sizeof(cx));
    r->sb = (cx*)calloc(r->NS, sizeof(cx));
    r->scr = (size_t)4 * (c->nx > c->ny ? c->nx : c->ny);
    r->scratch = (cx*)calloc(r->scr * (size_t)r->nthreads, sizeof(cx));
    for (int f = 0; f < 7; ++f)
        if (!*fields[f]) { cpu_destroy(r); return NULL; }
    for (int f = 0; f < 24; ++f)
        if (!r->t[f]) { cpu_destroy(r); return NULL; }
    if (!r->sa || !r->sb || !r->scratch) { cpu_destroy(r); return NULL; }
    /* initialize_fields_3d (3D:909-962): U = u_c (1 - z^2), v = w = p = 0,
     * the analytical perturbation (perturbation_analytical_simple.f90:24-133),
     * walls zeroed (3D:3253) */
    for (int k = 0; k < nz; ++k)
        for (size_t i = 0; i < r->pl; ++i) r->u[k * r->pl + i] = c->u_centerline * (1.0 - r->zpts[k] * r->zpts[k]);
    if (c->enable_perturbations && c->use_analytical_perturbations) {
        const double kx = 2.0 * pi * c->analytical_mode_x / c->xlen, ky = 2.0 * pi * c->analytical_mode_y / c->ylen;
        double cur = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            const double sc = pass == 0 ? 1.0 : (cur > 1.0e-12 ? c->perturbation_amplitude / cur : 0.0);
            if (pass == 1 && !(cur > 1.0e-12)) break;
            for (int k = 0; k < nz; ++k) {
                const double damp = 1.0 - r->zpts[k] * r->zpts[k];
                for (int j = 0; j < c->ny; ++j) {
                    const double y = j * c->ylen / c->ny;
                    for (int i = 0; i < c->nx; ++i) {
                        const double x = i * c->xlen / c->nx;
                        const double up = -ky * damp * (cos(ky * y) * sin(kx * x));
                        const double vp = kx * damp * (sin(ky * y) * cos(kx * x));
                        if (pass == 0) {
                            const double m = sqrt(up * up + vp * vp);
                            if (m > cur) cur = m;
                        } else if (k > 0 && k < nz - 1) {
                            const size_t o = k * r->pl + (size_t)j * c->nx + i;
                            r->u[o] += up * sc;
                            r->v[o] += vp * sc;
                        }
                    }
                }
            }
        }
        apply_bc(r);
    }
    r->current_pressure_gradient = c->target_pressure_gradient; /* 3D:623-635 */
    r->avg_pressure_gradient = c->target_pressure_gradient;
    return r;
}

void cpu_destroy(void* h) {
    cpu_run* r = (cpu_run*)h;
    if (!r) return;
    plan2d_free(&r->fp);
    free(r->zpts); free(r->zwts); free(r->d1); free(r->d2); free(r->xw); free(r->yw);
    free(r->u); free(r->v); free(r->w); free(r->p); free(r->gpx); free(r->gpy); free(r->gpz);
    for (int f = 0; f < 24; ++f) free(r->t[f]);
    free(r->sa); free(r->sb); free(r->scratch);
    free(r);
}

/* The loop body (3D:286-361) without IO, nsteps times.  0, or -1 if an
 * operator was singular (the reference stops in zgesv). */
int cpu_step(void* h, int nsteps) {
    cpu_run* r = (cpu_run*)h;
    for (int s = 0; s < nsteps; ++s) {
        r->istep += 1;
        r->time += r->c.dt;
        source_terms(r);
        if (viscous_step(r) || solve_pressure(r)) return -1;
        pressure_correction(r);
        apply_bc(r);
    }
    return 0;
}

/* u, v, w, p_total (N each, may be NULL); pi[7]: current dP/dx, U_b,
 * error, integral, previous error, sum, average */
void cpu_get_state(void* h, double* u, double* v, double* w, double* p, double* pi) {
    cpu_run* r = (cpu_run*)h;
    const size_t b = sizeof(double) * r->N;
    if (u) memcpy(u, r->u, b);
    if (v) memcpy(v, r->v, b);
    if (w) memcpy(w, r->w, b);
    if (p) memcpy(p, r->p, b);
    if (pi) {
        pi[0] = r->current_pressure_gradient; pi[1] = r->current_bulk_velocity; pi[2] = r->bulk_velocity_error;
        pi[3] = r->bulk_velocity_error_integral; pi[4] = r->bulk_velocity_error_prev;
        pi[5] = r->pressure_gradient_sum; pi[6] = r->avg_pressure_gradient;
    }
}

/* Replace u, v, w (and p_total, the wall-gradient fields when given). */
void cpu_set_state(void* h, const double* u, const double* v, const double* w, const double* p, const double* gpx,
                   const double* gpy) {
    cpu_run* r = (cpu_run*)h;
    const size_t b = sizeof(double) * r->N;
    if (u) memcpy(r->u, u, b);
    if (v) memcpy(r->v, v, b);
    if (w) memcpy(r->w, w, b);
    if (p) memcpy(r->p, p, b);
    if (gpx) memcpy(r->gpx, gpx, b);
    if (gpy) memcpy(r->gpy, gpy, b);
}

/* output_diagnostics_3d (3D:2094-2146): umax, vmax, wmax, energy, dP/dx, U_b
 * (method 2), dP/dx average, max divergence (check_divergence_3d) */
void cpu_diagnostics(void* h, double* out8) {
    cpu_run* r = (cpu_run*)h;
    double mu = 0, mv = 0, mw = 0, e = 0;
    const double fac = (r->c.xlen / r->nx) * (r->c.ylen / r->ny) * (r->ybar / 2.0);
    for (int k = 0; k < r->nz; ++k)
        for (size_t i = 0; i < r->pl; ++i) {
            const size_t o = k * r->pl + i;
            const double a = r->u[o], b = r->v[o], c = r->w[o];
            if (fabs(a) > mu) mu = fabs(a);
            if (fabs(b) > mv) mv = fabs(b);
            if (fabs(c) > mw) mw = fabs(c);
            e += 0.5 * (a * a + b * b + c * c) * fac * r->zwts[k];
        }
    out8[0] = mu; out8[1] = mv; out8[2] = mw;
    out8[3] = e / (r->c.xlen * r->c.ylen * r->ybar);
    out8[4] = r->current_pressure_gradient;
    out8[5] = r->c.flow_control_method == 2 ? bulk_velocity(r, r->u) : r->current_bulk_velocity;
    out8[6] = r->avg_pressure_gradient;
    derivatives(r, r->u, r->t[3], NULL, NULL);
    derivatives(r, r->v, NULL, r->t[4], NULL);
    derivatives(r, r->w, NULL, NULL, r->t[5]);
    double md = 0.0;
    for (size_t i = 0; i < r->N; ++i) {
        const double d = fabs(r->t[3][i] + r->t[4][i] + r->t[5][i]);
        if (d > md) md = d;
    }
    out8[7] = md;
}

int cpu_threads(void* h) { return ((cpu_run*)h)->nthreads; }

/* Raw 2D transforms of one plane, for checking the FFT restatement. */
int cpu_r2c_plane(int nx, int ny, const double* in, double* out_cx) {
    plan2d p;
    if (plan2d_init(&p, nx, ny)) return -1;
    cx* s = (cx*)malloc(sizeof(cx) * 4 * (nx > ny ? nx : ny));
    r2c_plane(&p, in, (cx*)out_cx, s);
    free(s);
    plan2d_free(&p);
    return 0;
}

int cpu_c2r_plane(int nx, int ny, const double* in_cx, double* out) {
    plan2d p;
    if (plan2d_init(&p, nx, ny)) return -1;
    const size_t n = (size_t)(nx / 2 + 1) * ny;
    cx* tmp = (cx*)malloc(sizeof(cx) * n);
    memcpy(tmp, in_cx, sizeof(cx) * n);
    cx* s = (cx*)malloc(sizeof(cx) * 4 * (nx > ny ? nx : ny));
    c2r_plane(&p, tmp, out, s);
    free(s);
    free(tmp);
    plan2d_free(&p);
    return 0;
}

/*
 * dns3d_capi.h -- C-ABI of the GB300 (sm_103a) 3D channel-flow time step.
 *
 * Drop-in for the time loop of DNS_pressure_BC_3D.f90 (chandc/F90_DNS).  The
 * reference step is five argument-less internal subroutines that share state
 * through host-associated arrays (DNS_pressure_BC_3D.f90:108-178, called at
 * :314-326).  Here that state lives on the GPU inside an opaque handle; the
 * five subroutines become five entry points with the same names and order, so
 * a Fortran driver binds them with ISO_C_BINDING and keeps its loop.
 *
 * Conventions
 *  - Every entry point returns an int status: DNS3D_OK (0) or a DNS3D_E_*
 *    code.  Nothing here exits, prints or throws (the reference `stop`s, e.g.
 *    DNS_pressure_BC_3D.f90:837-875, 1506, 1715-1718).
 *  - Host arrays are caller-owned, contiguous, Fortran order u(nx,ny,nz)
 *    (i fastest), i.e. C u[k][j][i]; k = 1 is the wall z = -1.  The library
 *    copies in and out; device state is library-owned and stays resident.
 *  - One host thread per handle.  Distinct handles are independent.
 */
#ifndef DNS3D_CAPI_H
#define DNS3D_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

#define DNS3D_OK 0
#define DNS3D_E_INVALID 1      /* bad argument or configuration value        */
#define DNS3D_E_OOM 2          /* device allocation failed                   */
#define DNS3D_E_SINGULAR 3     /* a per-mode operator could not be inverted  */
#define DNS3D_E_NONFINITE 4    /* NaN/Inf detected in the state              */
#define DNS3D_E_CUDA 5         /* CUDA runtime / launch error                */
#define DNS3D_E_UNSUPPORTED 6  /* grid size or option not supported          */
#define DNS3D_E_IO 7           /* input file could not be read / parsed      */
#define DNS3D_E_NODEVICE 8     /* no CUDA device                              */
#define DNS3D_E_TIMEOUT 9      /* a wait ran out of time                      */
#define DNS3D_E_CANCELLED 10   /* a served request was cancelled              */

#define DNS3D_PREC_FP64 0      /* plain FP64 path                            */
#define DNS3D_PREC_MIXED 1     /* FP32 nonlinear term and viscous increment;
                                  FP64 state, (0,0) mode, PI controller, wall
                                  rows, pressure projection and diagnostics  */

/* Namelist parameters of read_input_3d (DNS_pressure_BC_3D.f90:559-568,
 * defaults 571-603).  alpha, beta and ybar are derived (3D:740-742), the
 * read-but-unused ta, cs, u00, wavlen, cgstol, iform, iles are not carried. */
typedef struct dns3d_config {
    int nx, ny, nz;                    /* &grid nx_input, ny_input, nz_input */
    int istart, nsteps, nwrt, restart_write_freq;  /* &time_control */
    double dt;
    double re, xlen, ylen, u_centerline;            /* &simulation */
    int use_crank_nicolson;
    int flow_control_method;                        /* &flow_control: 1 or 2 */
    double target_pressure_gradient, target_bulk_velocity, controller_gain;
    int controller_update_freq;
    int enable_perturbations;                       /* &perturbations */
    double perturbation_amplitude;
    int zero_w_perturbations, use_analytical_perturbations;
    int analytical_mode_x, analytical_mode_y;
    int use_weak_form_divergence;                   /* &pressure_solver */
    int use_dealias_23_rule;                        /* &computational */
    /* 1 (default) = the reference's differentiation_matrix, which zeroes any
     * entry whose Lagrange denominator is <= 1e-15 (lgl_module.f90:247-251);
     * for nz >= 58 that is every off-diagonal entry and the pinned Poisson
     * mode is singular, so dns3d_create fails with DNS3D_E_SINGULAR, as the
     * reference stops in zgesv (3D:1715-1718).  0 = the same Lagrange formula
     * without that cutoff.  Read from &computational as an extension key. */
    int lgl_dmatrix_guard;
    int precision;                                  /* DNS3D_PREC_*        */
    int device;                                     /* CUDA device ordinal */
    /* Seed of the random solenoidal perturbation (enable_perturbations with
     * use_analytical_perturbations = 0, perturbation_module.f90:42-176).  The
     * reference seeds gfortran's random_number from the clock, so its runs
     * cannot be repeated; here a SplitMix64 stream started from this seed
     * supplies the uniform draws, in the reference's order.  Read from
     * &perturbations as an extension key. */
    long long perturbation_seed;
    /* Optional schemes (extension keys of &computational; the reference's 3D
     * solver has neither, its 2D solver has both):
     * convection_scheme 0 = the 3D step's single explicit evaluation of the
     *   nonlinear term (3D:1032-1098); 1 = jst4, the four-stage scheme of
     *   runge_kutta_convection (DNS_pressure_BC_2D.f90:931-1014) lifted to 3D:
     *   for a = 1/4, 1/3, 1/2 the stage state is u^n + a dt S(previous stage)
     *   with S the (filtered) rotational nonlinear term and the walls zeroed,
     *   and the step uses S of the last stage state (forcing added once).
     * linear_solver 0 = the per-mode Helmholtz and Poisson systems solved
     *   directly (the reference's zgesv); 1 = jacgs, Jacobi-preconditioned
     *   conjugate gradients (DNS_pressure_BC_2D.f90:2361-2476) on every
     *   non-pinned Poisson system and on the interior Helmholtz systems, FP64,
     *   at most 500 iterations, stopping when the residual 2-norm falls to
     *   cgstol times its initial value (a relative test: the spectra here are
     *   unnormalised sums).  FP64 precision only. */
    int convection_scheme;
    int linear_solver;
    double cgstol;                                  /* &simulation cgstol (default 1e-6, 3D:575) */
    /* Seeded white noise added to the initial u, v, w after the perturbation
     * (walls zeroed again): uniform in [-noise_amplitude, noise_amplitude),
     * from Philox4x32-10 (Salmon et al., SC'11) with key perturbation_seed and
     * counter (point index low, high, component, 0), top 53 bits of the first
     * two outputs.  Not a reference feature (the large-grid workload's
     * initial condition); 0 = none.  Extension key of &perturbations. */
    double noise_amplitude;
    /* Mixed precision only: 1 = one step of iterative refinement of every
     * mixed-precision Poisson solve (the residual of the FP32 solution formed
     * with the stiffness matrix in double-float arithmetic, the FP32
     * correction added), which brings the Galerkin residual of the system
     * solve_pressure_3d_standard solves (3D:1680-1714) from ~3e-6 to ~5e-12
     * of its right-hand side at 128x128x65; 0 (default) = the FP32 solve in
     * the eigenbasis alone, whose error is relative to each eigen-component
     * and so already small where the system is ill-conditioned.  The
     * refinement costs about 40% of a mixed step and does not reduce the
     * velocity error against FP64, which the FP32 transforms set.  Extension
     * key of &computational. */
    int poisson_refinement;
    int pad_;
} dns3d_config;

/* PI controller globals (DNS_pressure_BC_3D.f90:75-89). */
typedef struct dns3d_pi_state {
    double current_pressure_gradient;
    double current_bulk_velocity;
    double bulk_velocity_error;
    double bulk_velocity_error_integral;
    double bulk_velocity_error_prev;
    double pressure_gradient_sum;
    double avg_pressure_gradient;
    int pressure_gradient_count;
    int pad_;
} dns3d_pi_state;

/* Observables of output_diagnostics_3d (3D:2094-2146) and check_divergence_3d
 * (3D:2171-2190). */
typedef struct dns3d_diag {
    double umax, vmax, wmax, energy;
    double u_bulk, dpdx, dpdx_avg;
    double max_div;
    double time;
    int step;
    int pad_;
} dns3d_diag;

typedef struct dns3d_handle dns3d_handle;

/* Defaults of read_input_3d (3D:571-603). */
int dns3d_config_defaults(dns3d_config* cfg);

/* Parse a Fortran namelist input file with the eight groups of read_input_3d
 * (3D:606-616).  Unknown keys are ignored; missing groups keep defaults. */
int dns3d_config_read_namelist(const char* path, dns3d_config* cfg);

/* Grid/spectral setup, LGL operators, per-mode operators, device allocation
 * (setup_grid_3d 3D:728, setup_spectral_3d 3D:769, allocate_arrays_3d 3D:831,
 * setup_fftw3_plans_dns fftw3_dns_module.f90:60).  The state starts at the
 * initial condition of initialize_fields_3d (3D:909-962). */
int dns3d_create(const dns3d_config* cfg, dns3d_handle** out);
int dns3d_destroy(dns3d_handle* h);

/* initialize_fields_3d (3D:909-962) incl. the analytical perturbation
 * (perturbation_analytical_simple.f90:24-155); resets step and time. */
int dns3d_initialize_fields(dns3d_handle* h);

/* Copy state in/out.  Any pointer may be NULL (that field is left as is /
 * not returned).  gp*_w1/_w2 are the wall planes k=1 and k=nz of
 * grad_p_prev_x/_y (nx*ny each), the only part of those arrays the step
 * reads (3D:1325-1326).  In dns3d_set_state, if all four are NULL and
 * p_total is given, the wall gradients are recomputed from p_total (the
 * relation pressure_correction_3d leaves behind, 3D:1923). */
int dns3d_set_state(dns3d_handle* h, const double* u, const double* v, const double* w,
                    const double* p_total, const double* gpx_w1, const double* gpx_w2,
                    const double* gpy_w1, const double* gpy_w2, const dns3d_pi_state* pi);
int dns3d_get_state(dns3d_handle* h, double* u, double* v, double* w, double* p_total,
                    double* gpx_w1, double* gpx_w2, double* gpy_w1, double* gpy_w2,
                    dns3d_pi_state* pi);
int dns3d_set_clock(dns3d_handle* h, int step, double time);

/* The five subroutines of the time loop, in the reference's order
 * (DNS_pressure_BC_3D.f90:314-326). */
int dns3d_compute_source_terms(dns3d_handle* h);   /* 3D:1032-1148 */
int dns3d_viscous_step(dns3d_handle* h);           /* 3D:1285-1521 */
int dns3d_solve_pressure(dns3d_handle* h);         /* 3D:1631-1835 */
int dns3d_pressure_correction(dns3d_handle* h);    /* 3D:1903-1929 */
int dns3d_apply_boundary_conditions(dns3d_handle* h); /* 3D:1953-1972 */

/* nsteps passes of the loop body (3D:286-361 without IO): time += dt and the
 * five subroutines, fused and replayed as a CUDA graph. */
int dns3d_step(dns3d_handle* h, int nsteps);

/* Wait for all work queued on the handle's stream. */
int dns3d_synchronize(dns3d_handle* h);
/* Without waiting: *done = 1 if all work queued on the handle has completed,
 * else 0 (for a driver that overlaps runs, e.g. the request server). */
int dns3d_query(dns3d_handle* h, int* done);

/* output_diagnostics_3d observables plus check_divergence_3d's max |div u|. */
int dns3d_diagnostics(dns3d_handle* h, dns3d_diag* out);
/* The two reference routines one at a time, for a driver that calls them on
 * the reference's schedule (every nwrt steps, every 50 steps, 3D:329-344):
 * output_diagnostics_3d (3D:2094-2146) -- *out as dns3d_diagnostics gives it,
 * with max_div = 0 -- and check_divergence_3d (3D:2171-2190). */
int dns3d_output_diagnostics(dns3d_handle* h, dns3d_diag* out);
int dns3d_check_divergence(dns3d_handle* h, double* max_div);

/* Accuracy of the last pressure solve: the relative residual max|b - P phi| /
 * max|b| of the Galerkin Poisson system that solve_pressure_3d_standard
 * builds and solves per mode (3D:1680-1714; the weak form 1793-1816):
 * P = -S - diag(k^2 w ybar/2), b from the handle's u*, v*, w* and phi its
 * solution, mode (0,0) without its pinned row and column.  This is the
 * divergence the projection controls; the collocation max|div u| of
 * check_divergence_3d also carries the wall rows the boundary conditions
 * overwrite after the projection.  Valid after a step (or after the
 * five-stage calls up to dns3d_pressure_correction).  No counterpart in the
 * reference. */
int dns3d_projection_residual(dns3d_handle* h, double* rel);

/* Measurement helpers (no counterpart in the reference, whose only timing is
 * cpu_time around each step, 3D:287-360).
 * dns3d_step_timed: dns3d_step with CUDA events recorded on the handle's
 * stream around the nsteps graph replays; waits and returns the elapsed ms.
 * dns3d_profile_kernels: runs nsteps loop bodies launch by launch with an
 * event between consecutive kernels and returns, per kernel name, the launch
 * count and total device ms (names are static strings). */
typedef struct dns3d_kernel_time {
    const char* name;
    int launches;
    int pad_;
    double total_ms;
} dns3d_kernel_time;
int dns3d_step_timed(dns3d_handle* h, int nsteps, double* elapsed_ms);
int dns3d_profile_kernels(dns3d_handle* h, int nsteps, dns3d_kernel_time* out, int cap, int* n);
/* Kernel launches one dns3d_step issues per time step. */
int dns3d_launches_per_step(dns3d_handle* h, int* n);
/* Dense FP64 FMA throughput of `device` in TFLOP/s (FMA = 2 flops), timed with
 * CUDA events: the peak that bounds the FP64 kernels. */
int dns3d_measure_fp64_tflops(int device, double* tflops);
/* Self-check of the library's integer-pipe conversions against the hardware
 * ones on n pseudo-random values: FP64<->FP32 (the mixed-precision kernels)
 * over the normal float range, and int64 -> FP64 with a power-of-two scaling
 * (the fixed-point transforms and the tensor-core epilogues) over every
 * integer bit length and scalings into and out of the FP64 range:
 * *mismatches = 0 expected. */
int dns3d_check_conversions(int device, long long n, unsigned long long* mismatches);

/* Flow statistics without any device allocation.  No counterpart in the
 * reference.  For callers that cannot let a library allocate device memory
 * (a driver that reserves nearly all HBM for its own pool, a job with a fixed
 * memory budget) and so cannot create a handle just to read diagnostics.
 * Given caller-owned device arrays u, v, w (nx*ny*nz doubles each, the layout
 * of dns3d_get_state), writes to the caller-owned device buffer out4:
 *   out4[0..2] = max|u|, max|v|, max|w|,
 *   out4[3]    = kinetic energy, as dns3d_diagnostics() reports them.
 * A NaN in out4 means a non-finite value in the fields (the maxima keep NaN).
 * Runs on the calling thread's current device, asynchronously on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  Its scratch is a fixed
 * 32 KB array inside the library, present on every GPU that loads it until
 * the process exits; it allocates nothing.  The first call on a device looks
 * up that array's device address (make that first call before any stream
 * capture); that address is kept per device ordinal for the life of the
 * process, so it does not survive cudaDeviceReset() or a change of context on
 * the device.  All calls share the array, so calls that overlap on the GPU
 * race.
 * nz above DNS3D_NOALLOC_MAX_NZ is rejected with DNS3D_E_UNSUPPORTED. */
#define DNS3D_NOALLOC_MAX_NZ 129
int dns3d_flow_stats_noalloc(const double* u, const double* v, const double* w, int nx, int ny,
                             int nz, double* out4, void* stream);

/* Batches: joint stepping of independent runs (any mix of grids, parameters
 * and precisions).  No counterpart in the reference, which runs one channel
 * per process.  Runs whose options allow it (the default convection scheme
 * and solver, transform lengths with compile-time kernels, fewer than 2^20
 * grid points -- larger runs fill the GPU with their own launches) advance in
 * ragged launches: each of the ten stages of a step (vorticity with the PI
 * update, four plane-transform passes, the products, viscous, pressure,
 * projection, walls) is ONE kernel launch over the mode tiles / transform
 * columns of all such runs of one precision and kernel variant (which stages
 * run their tensor-core forms), whatever their nx, ny, nz, with
 * every run's arithmetic that of its own launches (bitwise the same results);
 * the mixed form adds one launch each for the FP64 mode (0,0) viscous and
 * pressure solves, beside the tiles.  Other runs are stepped by their own
 * launches beside them.  One step is one CUDA graph;
 * DNS3D_BATCH_TUNE times the stage tile widths for this set of runs when the
 * batch is created (the runs' PI states are restored afterwards).  The
 * handles stay owned by the caller and must outlive the batch; the batch
 * orders itself after work already queued on each run's stream, and later
 * work on those streams after the batch's steps. */
typedef struct dns3d_batch dns3d_batch;
#define DNS3D_BATCH_TUNE 1
int dns3d_batch_create(dns3d_handle* const* runs, int nruns, int flags, dns3d_batch** out);
/* Queues nsteps steps of every run (returns before they finish). */
int dns3d_batch_step(dns3d_batch* b, int nsteps);
int dns3d_batch_synchronize(dns3d_batch* b);
/* Without waiting: *done = 1 if the batch's queued steps have completed. */
int dns3d_batch_query(dns3d_batch* b, int* done);
/* Kernel launches per step of the whole batch, and how many runs are in
 * ragged launches (the rest use their own). */
int dns3d_batch_info(dns3d_batch* b, int* launches_per_step, int* ragged_runs);
int dns3d_batch_destroy(dns3d_batch* b);

/* Ensembles: a batch that owns its runs, created from configs.  Runs are
 * numbered 0..nruns-1 in config order; the stage tile widths are tuned for the
 * ensemble at its first step unless DNS3D_AUTOTUNE=0. */
typedef struct dns3d_ensemble dns3d_ensemble;
int dns3d_ensemble_create(const dns3d_config* cfgs, int nruns, dns3d_ensemble** out);
int dns3d_ensemble_destroy(dns3d_ensemble* e);
int dns3d_ensemble_size(dns3d_ensemble* e, int* nruns);
/* The handle of run i (state transfer, diagnostics); owned by the ensemble. */
int dns3d_ensemble_run(dns3d_ensemble* e, int i, dns3d_handle** h);
/* Advances every run nsteps steps; returns when they are done. */
int dns3d_ensemble_step(dns3d_ensemble* e, int nsteps);
/* As dns3d_ensemble_step, bracketed by CUDA events; waits, returns device ms. */
int dns3d_ensemble_step_timed(dns3d_ensemble* e, int nsteps, double* elapsed_ms);
/* As dns3d_batch_info for the ensemble's batch (created at the first step). */
int dns3d_ensemble_info(dns3d_ensemble* e, int* launches_per_step, int* ragged_runs);

/* Serving: continuous batching of requested runs on one GPU.  No counterpart
 * in the reference.  A worker thread owned by the server admits requests in
 * FIFO order while their device footprint fits under max_bytes and fewer than
 * max_runs are running, advances all running requests steps_per_round steps
 * per round (the runs taking a full round as one dns3d_batch, rebuilt when
 * that set changes; a run's shorter last round on its own stream beside it),
 * and frees a run's device memory as soon as it completes
 * (DNS3D_SERVER_BATCH=0 in the environment: every run on its own stream).
 * Times are seconds since server creation.  dns3d_server_destroy cancels
 * queued and running requests. */
#define DNS3D_REQ_QUEUED 0
#define DNS3D_REQ_RUNNING 1
#define DNS3D_REQ_DONE 2
#define DNS3D_REQ_FAILED 3
typedef struct dns3d_server dns3d_server;
typedef struct dns3d_server_opts {
    unsigned long long max_bytes;  /* device memory budget (default 160 GiB) */
    int max_runs;                  /* concurrent runs (default 256)           */
    int steps_per_round;           /* steps per run between waits (default 10)*/
    int device;
    int pad_;
} dns3d_server_opts;
typedef struct dns3d_request_info {
    int status;                    /* DNS3D_REQ_*                             */
    int error;                     /* DNS3D_OK or the failing status          */
    int steps_done, nsteps;
    unsigned long long bytes;      /* admitted footprint                      */
    double t_submit, t_start, t_finish;  /* -1 if not reached                 */
    dns3d_diag diag;               /* final diagnostics (when done)           */
} dns3d_request_info;
typedef struct dns3d_server_stats {
    int queued, running;
    unsigned long long bytes_in_use;
    unsigned long long point_steps_done;  /* of completed requests           */
    double uptime_s;
} dns3d_server_stats;
int dns3d_server_opts_defaults(dns3d_server_opts* opts);
int dns3d_server_create(const dns3d_server_opts* opts, dns3d_server** out);
/* Queue a run of `nsteps` steps of cfg (from its initial condition); with
 * keep_state the final u, v, w, p_total are kept for
 * dns3d_server_result_state until dns3d_server_release. */
int dns3d_server_submit(dns3d_server* s, const dns3d_config* cfg, int nsteps, int keep_state,
                        long long* request_id);
int dns3d_server_poll(dns3d_server* s, long long request_id, dns3d_request_info* info);
/* Wait until the request is done or failed (timeout_s < 0: no limit);
 * DNS3D_E_TIMEOUT if the time ran out. */
int dns3d_server_wait(dns3d_server* s, long long request_id, double timeout_s, dns3d_request_info* info);
int dns3d_server_result_state(dns3d_server* s, long long request_id, double* u, double* v, double* w,
                              double* p_total);
int dns3d_server_release(dns3d_server* s, long long request_id);
int dns3d_server_get_stats(dns3d_server* s, dns3d_server_stats* stats);
int dns3d_server_destroy(dns3d_server* s);

/* Restart files in the reference's format (write_restart_file_3d /
 * read_restart_file_3d, DNS_pressure_BC_3D.f90:2976-3209): Fortran stream
 * unformatted, no record markers, little-endian:
 *   'DNS3D_RESTART_v1.0' (18 bytes); istep (int32), time, dt (f64);
 *   nx, ny, nz (int32); re, alpha, beta (f64); u, v, w, un, vn, wn, p_total
 *   (f64, u(nx,ny,nz) order each); current_pressure_gradient,
 *   current_bulk_velocity, bulk_velocity_error_integral,
 *   bulk_velocity_error_prev (f64).
 * The two host functions encode and decode a file from caller arrays (no GPU);
 * NULL arrays are written as zeros / skipped on read.  A grid mismatch on read
 * returns DNS3D_E_INVALID (the reference then ignores the file); a file that
 * ends before the four PI scalars keeps them at their defaults, as the
 * reference does. */
typedef struct dns3d_restart_header {
    int istep;
    int nx, ny, nz;
    double time, dt;
    double re, alpha, beta;
} dns3d_restart_header;
int dns3d_restart_write(const char* path, const dns3d_restart_header* hdr, const double* u, const double* v,
                        const double* w, const double* un, const double* vn, const double* wn,
                        const double* p_total, const dns3d_pi_state* pi);
/* hdr->nx, ny, nz give the expected grid on entry; the rest is filled in.
 * pi fields not in the file (sum, count, average) are left unchanged. */
int dns3d_restart_read(const char* path, dns3d_restart_header* hdr, double* u, double* v, double* w,
                       double* un, double* vn, double* wn, double* p_total, dns3d_pi_state* pi);
/* Handle level: save the current state as a restart file (un, vn, wn are
 * written equal to u, v, w: the state at the start of a step, which is what
 * the reference's in-loop writes record, 3D:300-308); load one into the
 * handle.  Loading sets u, v, w, p_total and the four PI scalars and leaves
 * the wall gradients grad_p_prev at zero, as the reference's restart does
 * (it never restores them, 3D:957, 3057-3209). */
int dns3d_save_restart(dns3d_handle* h, const char* path, int istep, double time);
int dns3d_load_restart(dns3d_handle* h, const char* path, int* istep, double* time);
/* The configuration the handle was created with. */
int dns3d_get_config(dns3d_handle* h, dns3d_config* cfg);
/* Tile autotuner.  The mode-tile kernels (vorticity, viscous, pressure,
 * correction, divergence and their mixed forms; DNS3D_TILE_KERNELS of them, in
 * that order) process a number of mode columns per CTA.  dns3d_create times
 * the candidate widths 4..64 of the kernels the handle runs on its own buffers
 * and keeps the fastest, remembered per (grid, precision, device) for the
 * process; set DNS3D_AUTOTUNE=0 in the environment to keep the built-in
 * widths.  Results do not depend on the widths (every output is one thread's
 * fixed-order sum).  dns3d_autotune re-runs the tuning (force = 1 ignores the
 * remembered choice, force < 0 only reports) and reports the widths in use
 * (tiles[k], k < ntiles); dns3d_set_tiles sets
 * them (0 = built-in), DNS3D_E_INVALID if one does not fit the kernel's
 * shared memory. */
#define DNS3D_TILE_KERNELS 8
int dns3d_autotune(dns3d_handle* h, int force, int* tiles, int ntiles);
int dns3d_set_tiles(dns3d_handle* h, const int* tiles, int ntiles);

/* The handle's step counter and time (dns3d_set_clock, advanced by dns3d_step). */
int dns3d_get_clock(dns3d_handle* h, int* step, double* time);
/* LGL nodes (z, ascending from -1) and weights of lgl_module.f90:30-80. */
int dns3d_lgl_nodes_weights(int nz, double* z, double* w);

/* ---- Flow statistics and the reference's output files ----------------------
 * The numbers of write_time_series_data, write_flow_statistics and
 * write_spanwise_averaged_profile (DNS_pressure_BC_3D.f90:2702-2952),
 * reduced from the device state at the handle's clock. */
typedef struct dns3d_flow_stats {
    double umax, vmax, wmax;     /* max |u|, |v|, |w|                                  */
    double energy;               /* mean kinetic energy with LGL weights (3D:2710-2730) */
    double bulk_velocity;        /* method 2: calculate_bulk_velocity_3d (3D:2434-2464);
                                    otherwise sum u*zwts/(nx*ny)/2 (3D:2874-2889)     */
    double dpdx, dpdx_avg;       /* current and running-average dP/dx                 */
    double wall_shear_lower;     /* (1/Re) * plane mean of (u_2 - u_1)/(z_2 - z_1)     */
    double wall_shear_upper;     /* (1/Re) * plane mean of (u_nz - u_nz-1)/(z_nz - z_nz-1) (3D:2891-2921) */
    double friction_velocity_avg;/* sqrt((|tau_lower| + |tau_upper|)/2) (3D:2948)      */
    double re_tau;               /* friction_velocity_avg * Re (3D:2949)              */
    double time;
    int step;
    int flow_control_method;
} dns3d_flow_stats;
/* u_avg, v_avg, w_avg (nz each, may be NULL): plane means per level k. */
int dns3d_flow_statistics(dns3d_handle* h, dns3d_flow_stats* out, double* u_avg, double* v_avg, double* w_avg);

/* Host file writers in the reference's formats (no GPU).  `dir` is an
 * existing directory (the reference's timestamped output directory is the
 * caller's choice).
 *  - output_init: output_time_series.dat and flow_statistics.dat with their
 *    headers (initialize_output_files, 3D:2667-2694);
 *  - time_series_row: one '(I8,7(ES15.6))' row (method 2: average dP/dx and
 *    U_bulk) or '(I8,6(ES15.6))' row (current dP/dx) appended to
 *    output_time_series.dat, which must exist (3D:2736-2745);
 *  - flow_statistics: flow_statistics.dat replaced (3D:2925-2951);
 *  - spanwise_profile: spanwise_profile_NNNNN.dat (3D:2808-2838);
 *  - velocity_snapshot: velocity_field_NNNNN.dat, '(3I6,6ES15.6)' per point,
 *    k outermost, i fastest (3D:2765-2786);
 *  - simulation_summary: simulation_summary.txt (3D:2594-2659), start time
 *    from the local clock. */
int dns3d_output_init(const char* dir);
int dns3d_output_time_series_row(const char* dir, const dns3d_flow_stats* st);
int dns3d_output_flow_statistics(const char* dir, const dns3d_flow_stats* st);
int dns3d_output_spanwise_profile(const char* dir, int istep, double time, int nz, const double* z,
                                  const double* u_avg, const double* v_avg, const double* w_avg);
int dns3d_output_velocity_snapshot(const char* dir, int istep, double time, int nx, int ny, int nz, double xlen,
                                   double ylen, const double* z, const double* u, const double* v, const double* w);
int dns3d_output_simulation_summary(const char* dir, const dns3d_config* cfg, const char* input_filename,
                                    const char* output_directory, const char* restart_filename, int restarted,
                                    int restart_step, double restart_time);
/* Handle level, the reference's subroutine names: reduce the state on the
 * device and write the file at the handle's step and time. */
int dns3d_write_time_series_data(dns3d_handle* h, const char* dir);
int dns3d_write_flow_statistics(dns3d_handle* h, const char* dir);
int dns3d_write_spanwise_averaged_profile(dns3d_handle* h, const char* dir);
int dns3d_write_velocity_field_snapshot(dns3d_handle* h, const char* dir);

/* Device bytes held by a handle for a given config (admission control). */
int dns3d_footprint_bytes(const dns3d_config* cfg, unsigned long long* bytes);

const char* dns3d_strerror(int code);

/* Last CUDA error text recorded on the handle ("" if none). */
const char* dns3d_last_error(dns3d_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* DNS3D_CAPI_H */

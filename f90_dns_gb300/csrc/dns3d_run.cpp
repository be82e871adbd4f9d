// dns3d_run -- the reference program's driver loop over the GPU step.
//
// Mirrors `program dns_3d` of DNS_pressure_BC_3D.f90 (chandc/F90_DNS) around
// the time step: read the input file's namelists (read_input_3d, 3D:554-708),
// set up and initialise the fields (3D:184-206), then for istep = 1..nsteps
// advance time and call the five step subroutines in order (3D:286-326),
// print the diagnostics line every nwrt steps (output_diagnostics_3d,
// 3D:2134-2143) and the divergence every 50 steps (check_divergence_3d,
// 3D:2171-2190).  Like the reference it writes, into its output directory,
// simulation_summary.txt, output_time_series.dat and flow_statistics.dat
// every nwrt steps, velocity_field_NNNNN.dat and spanwise_profile_NNNNN.dat
// every 10*nwrt steps (3D:329-339), and restart.dat every restart_write_freq
// steps (at the start of the step, 3D:300-308) and after the last step
// (3D:367).  Timing summaries are not printed.
//
// The output directory is <input base name>_<YYYYMMDD_HHMMSS> in the working
// directory, as the reference's create_output_directory (3D:2557-2586), or
// the directory named by DNS3D_OUTPUT_DIR; DNS3D_OUTPUT_DIR=none writes no
// files.
//
// usage: dns3d_run [input_file]      (default input_3d.dat, as the reference)
// exit status: 0 on success, 1 on a library error (the reference `stop`s).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <sys/stat.h>

#include "dns3d_capi.h"

namespace {

// Fortran ES12.4: " d.ddddE+xx" right-aligned in 12 characters.
void es12_4(char* out, double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.4E", v);
    std::snprintf(out, 16, "%12s", buf);
}

// Fortran E12.4: " 0.ddddE+xx" right-aligned in 12 characters.
void e12_4(char* out, double v) {
    char buf[40];
    if (v == 0.0 || !std::isfinite(v)) {
        std::snprintf(buf, sizeof buf, v == 0.0 ? "0.0000E+00" : "%g", v);
    } else {
        int e = (int)std::floor(std::log10(std::fabs(v))) + 1;
        double m = std::fabs(v) / std::pow(10.0, e);
        char mb[32];
        std::snprintf(mb, sizeof mb, "%.4f", m);
        if (std::strcmp(mb, "1.0000") == 0) {
            e += 1;
            std::snprintf(mb, sizeof mb, "%.4f", m / 10.0);
        }
        std::snprintf(buf, sizeof buf, "%s%sE%c%02d", v < 0 ? "-" : "", mb, e < 0 ? '-' : '+', std::abs(e));
    }
    std::snprintf(out, 16, "%12s", buf);
}

// create_output_directory (3D:2557-2586): base name of the input file up to
// ".dat", then _YYYYMMDD_HHMMSS.
std::string output_directory(const char* input) {
    std::string base = input;
    const size_t dat = base.find(".dat");
    if (dat != std::string::npos) base = base.substr(0, dat);
    const std::time_t now = std::time(nullptr);
    std::tm t{};
    localtime_r(&now, &t);
    char ts[32];
    std::snprintf(ts, sizeof ts, "_%04d%02d%02d_%02d%02d%02d", t.tm_year + 1900, t.tm_mon + 1, t.tm_mday, t.tm_hour,
                  t.tm_min, t.tm_sec);
    return base + ts;
}

bool make_dirs(const std::string& path) {  // mkdir -p
    for (size_t i = 1; i <= path.size(); ++i)
        if (i == path.size() || path[i] == '/') {
            const std::string p = path.substr(0, i);
            struct stat st;
            if (stat(p.c_str(), &st) != 0 && mkdir(p.c_str(), 0755) != 0) return false;
        }
    return true;
}

int check(int rc, const char* where, dns3d_handle* h) {
    if (rc == DNS3D_OK) return 0;
    std::fprintf(stderr, " ERROR in %s: %s%s%s\n", where, dns3d_strerror(rc), h ? ": " : "",
                 h ? dns3d_last_error(h) : "");
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    const char* input = argc > 1 ? argv[1] : "input_3d.dat";
    dns3d_config cfg;
    dns3d_config_defaults(&cfg);
    if (dns3d_config_read_namelist(input, &cfg) != DNS3D_OK) {
        std::printf(" WARNING: Could not open input file: %s\n Using default parameters\n", input);
        dns3d_config_defaults(&cfg);
    } else {
        std::printf(" Input read from %s\n", input);
    }
    if (const char* dev = std::getenv("DNS3D_DEVICE")) cfg.device = std::atoi(dev);
    std::printf(" Grid: %d×%d×%d\n", cfg.nx, cfg.ny, cfg.nz);

    dns3d_handle* h = nullptr;
    if (check(dns3d_create(&cfg, &h), "dns3d_create", nullptr)) return 1;

    const char* od_env = std::getenv("DNS3D_OUTPUT_DIR");
    const bool files = !(od_env && std::strcmp(od_env, "none") == 0);
    const std::string od = od_env && *od_env && files ? std::string(od_env) : output_directory(input);
    const std::string restart_path = od + "/restart.dat";
    if (files) {
        if (!make_dirs(od)) {
            std::fprintf(stderr, " ERROR: cannot create output directory %s\n", od.c_str());
            return 1;
        }
        std::printf(" Output directory created:\n   %s\n", od.c_str());
        if (check(dns3d_output_init(od.c_str()), "initialize_output_files", h) ||
            check(dns3d_output_simulation_summary(od.c_str(), &cfg, input, od.c_str(), "restart.dat", 0, 0, 0.0),
                  "write_simulation_summary", h))
            return 1;
    }

    dns3d_diag d;
    double max_div = 0.0;
    if (check(dns3d_check_divergence(h, &max_div), "check_divergence_3d", h)) return 1;
    char dv[16];
    e12_4(dv, max_div);
    std::printf(" Step %6d, Max divergence: %s\n", 0, dv);

    double time = 0.0;
    char a[5][16];
    for (int istep = 1; istep <= cfg.nsteps; ++istep) {
        time = time + cfg.dt;
        if (files && cfg.restart_write_freq > 0 && istep % cfg.restart_write_freq == 0 &&
            check(dns3d_save_restart(h, restart_path.c_str(), istep, time), "write_restart_file_3d", h))
            return 1;
        dns3d_set_clock(h, istep, time);
        if (check(dns3d_compute_source_terms(h), "compute_source_terms_3d", h) ||
            check(dns3d_viscous_step(h), "viscous_step_3d", h) ||
            check(dns3d_solve_pressure(h), "solve_pressure_3d", h) ||
            check(dns3d_pressure_correction(h), "pressure_correction_3d", h) ||
            check(dns3d_apply_boundary_conditions(h), "apply_boundary_conditions_3d", h))
            return 1;
        const bool wrt = cfg.nwrt > 0 && istep % cfg.nwrt == 0;
        const bool div = istep % 50 == 0;
        if (wrt && check(dns3d_output_diagnostics(h, &d), "output_diagnostics_3d", h)) return 1;
        if (wrt) {
            es12_4(a[0], d.umax);
            es12_4(a[1], d.vmax);
            es12_4(a[2], d.wmax);
            es12_4(a[3], d.energy);
            es12_4(a[4], d.dpdx);
            if (cfg.flow_control_method == 2) {
                char ub[16], av[16];
                std::snprintf(ub, sizeof ub, "%8.5f", d.u_bulk);
                es12_4(av, d.dpdx_avg);
                std::printf(" Step %6d, t=%12.6f, |u|max=%s, |v|max=%s, |w|max=%s, E=%s, dP/dx=%s, U_bulk=%s, "
                            "dP/dx_avg=%s\n", istep, time, a[0], a[1], a[2], a[3], a[4], ub, av);
            } else {
                std::printf(" Step %6d, t=%12.6f, |u|max=%s, |v|max=%s, |w|max=%s, E=%s, dP/dx=%s\n", istep,
                            time, a[0], a[1], a[2], a[3], a[4]);
            }
        }
        if (wrt && files) {
            if (check(dns3d_write_time_series_data(h, od.c_str()), "write_time_series_data", h) ||
                check(dns3d_write_flow_statistics(h, od.c_str()), "write_flow_statistics", h))
                return 1;
            if (istep % (10 * cfg.nwrt) == 0) {
                if (check(dns3d_write_velocity_field_snapshot(h, od.c_str()), "write_velocity_field_snapshot", h) ||
                    check(dns3d_write_spanwise_averaged_profile(h, od.c_str()), "write_spanwise_averaged_profile", h))
                    return 1;
                std::printf(" Velocity field snapshot written: velocity_field_%05d.dat\n", istep);
                std::printf(" Spanwise profile written: spanwise_profile_%05d.dat\n", istep);
            }
        }
        if (div) {
            if (check(dns3d_check_divergence(h, &max_div), "check_divergence_3d", h)) return 1;
            e12_4(dv, max_div);
            std::printf(" Step %6d, Max divergence: %s\n", istep, dv);
        }
    }
    if (files && check(dns3d_save_restart(h, restart_path.c_str(), cfg.nsteps, time), "write_restart_file_3d", h))
        return 1;
    std::printf(" Time integration completed successfully!\n");
    dns3d_destroy(h);
    return 0;
}

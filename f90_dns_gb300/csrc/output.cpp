// Output files of the reference's time loop, in its text formats
// (DNS_pressure_BC_3D.f90:2594-2952): output_time_series.dat,
// flow_statistics.dat, spanwise_profile_NNNNN.dat,
// velocity_field_NNNNN.dat and simulation_summary.txt.
//
// The file writers are host code over plain arrays and a dns3d_flow_stats
// record; the handle-level entry points (the reference's subroutine names)
// take the statistics from dns3d_flow_statistics, which reduces the device
// state, and the fields from dns3d_get_state.
//
// Numbers are written with the Fortran edit descriptors the reference uses
// (ESw.d, Fw.d, Iw, I0), as gfortran renders them: ESw.d is one nonzero
// digit, d decimals and a two-digit exponent "E+dd" (three digits without
// the letter when |exponent| > 99), right-aligned; a field too narrow for
// the value is filled with '*'; NaN and infinities are spelt "NaN",
// "Infinity", "-Infinity" where they fit, else "Inf", "-Inf".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "dns3d_capi.h"

namespace {

std::string right(const std::string& s, int w) {
    if ((int)s.size() > w) return std::string(w, '*');
    return std::string(w - s.size(), ' ') + s;
}

std::string nonfinite(double v, int w) {
    if (std::isnan(v)) return right("NaN", w);
    if (w >= (v < 0 ? 9 : 8)) return right(v < 0 ? "-Infinity" : "Infinity", w);
    return right(v < 0 ? "-Inf" : "Inf", w);
}

// Fortran ESw.d
std::string fmt_es(double v, int w, int d) {
    if (!std::isfinite(v)) return nonfinite(v, w);
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*E", d, v);
    char* e = std::strchr(buf, 'E');
    const int ex = std::atoi(e + 1);
    if (ex > 99 || ex < -99) std::snprintf(e, sizeof buf - (e - buf), "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
    return right(buf, w);
}

// Fortran Fw.d
std::string fmt_f(double v, int w, int d) {
    if (!std::isfinite(v)) return nonfinite(v, w);
    char buf[512];
    std::snprintf(buf, sizeof buf, "%.*f", d, v);
    return right(buf, w);
}

// Fortran Iw
std::string fmt_i(long long v, int w) { return right(std::to_string(v), w); }

struct File {
    FILE* f = nullptr;
    File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
    void line(const std::string& s) { std::fputs((s + "\n").c_str(), f); }
    bool close() {
        const bool ok = f && std::fflush(f) == 0 && !std::ferror(f);
        if (f) std::fclose(f);
        f = nullptr;
        return ok;
    }
};

std::string join(const char* dir, const std::string& name) {
    std::string p = dir && *dir ? dir : ".";
    return p + "/" + name;
}

std::string numbered(const char* stem, int istep) {  // '(A,I5.5,A)'
    char b[64];
    if (istep < 0 || istep > 99999) std::snprintf(b, sizeof b, "%s*****.dat", stem);
    else std::snprintf(b, sizeof b, "%s%05d.dat", stem, istep);
    return b;
}

}  // namespace

extern "C" {

int dns3d_output_init(const char* dir) {
    // initialize_output_files, 3D:2667-2694 (directory creation is the caller's)
    {
        File f(join(dir, "output_time_series.dat"), "w");
        if (!f.f) return DNS3D_E_IO;
        f.line("# DNS 3D Time Series Data");
        f.line("# Columns: step, time, u_max, v_max, w_max, energy, pressure_gradient, bulk_velocity");
        if (!f.close()) return DNS3D_E_IO;
    }
    File f(join(dir, "flow_statistics.dat"), "w");
    if (!f.f) return DNS3D_E_IO;
    f.line("# DNS 3D Flow Statistics Summary");
    f.line("# Updated periodically during simulation");
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_output_time_series_row(const char* dir, const dns3d_flow_stats* st) {
    // write_time_series_data, 3D:2736-2745: '(I8,7(ES15.6))' for method 2
    // (average dP/dx and U_bulk), '(I8,6(ES15.6))' otherwise (current dP/dx).
    // The file must exist (the reference opens it status='old').
    if (!st) return DNS3D_E_INVALID;
    const std::string path = join(dir, "output_time_series.dat");
    {
        File probe(path, "r");
        if (!probe.f) return DNS3D_E_IO;
    }
    File f(path, "a");
    if (!f.f) return DNS3D_E_IO;
    std::string s = fmt_i(st->step, 8) + fmt_es(st->time, 15, 6) + fmt_es(st->umax, 15, 6) +
                    fmt_es(st->vmax, 15, 6) + fmt_es(st->wmax, 15, 6) + fmt_es(st->energy, 15, 6);
    if (st->flow_control_method == 2)
        s += fmt_es(st->dpdx_avg, 15, 6) + fmt_es(st->bulk_velocity, 15, 6);
    else
        s += fmt_es(st->dpdx, 15, 6);
    f.line(s);
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_output_flow_statistics(const char* dir, const dns3d_flow_stats* st) {
    // write_flow_statistics, 3D:2925-2951 (the file is replaced each time)
    if (!st) return DNS3D_E_INVALID;
    File f(join(dir, "flow_statistics.dat"), "w");
    if (!f.f) return DNS3D_E_IO;
    f.line("# DNS 3D Flow Statistics Summary");
    f.line("# Time step: " + std::to_string(st->step));
    f.line("# Time: " + fmt_f(st->time, 12, 6));
    f.line("");
    f.line("# Maximum velocities:");
    f.line("u_max = " + fmt_es(st->umax, 15, 6));
    f.line("v_max = " + fmt_es(st->vmax, 15, 6));
    f.line("w_max = " + fmt_es(st->wmax, 15, 6));
    f.line("");
    f.line("# Energy and bulk flow:");
    f.line("kinetic_energy = " + fmt_es(st->energy, 15, 6));
    f.line("bulk_velocity = " + fmt_es(st->bulk_velocity, 15, 6));
    f.line("pressure_gradient = " + fmt_es(st->flow_control_method == 2 ? st->dpdx_avg : st->dpdx, 15, 6));
    f.line("");
    f.line("# Wall shear stress:");
    f.line("tau_wall_lower = " + fmt_es(st->wall_shear_lower, 15, 6));
    f.line("tau_wall_upper = " + fmt_es(st->wall_shear_upper, 15, 6));
    f.line("friction_velocity_avg = " + fmt_es(st->friction_velocity_avg, 15, 6));
    f.line("re_tau = " + fmt_es(st->re_tau, 15, 6));
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_output_spanwise_profile(const char* dir, int istep, double time, int nz, const double* z,
                                  const double* u_avg, const double* v_avg, const double* w_avg) {
    // write_spanwise_averaged_profile, 3D:2808-2838: '(I6,4ES15.6)' per level
    if (nz < 1 || !z || !u_avg || !v_avg || !w_avg) return DNS3D_E_INVALID;
    File f(join(dir, numbered("spanwise_profile_", istep)), "w");
    if (!f.f) return DNS3D_E_IO;
    f.line("# DNS 3D Spanwise-Averaged Velocity Profile");
    f.line("# Time step: " + std::to_string(istep));
    f.line("# Time: " + fmt_f(time, 12, 6));
    f.line("# Columns: k, z, u_avg, v_avg, w_avg");
    for (int k = 0; k < nz; ++k)
        f.line(fmt_i(k + 1, 6) + fmt_es(z[k], 15, 6) + fmt_es(u_avg[k], 15, 6) + fmt_es(v_avg[k], 15, 6) +
               fmt_es(w_avg[k], 15, 6));
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_output_velocity_snapshot(const char* dir, int istep, double time, int nx, int ny, int nz, double xlen,
                                   double ylen, const double* z, const double* u, const double* v, const double* w) {
    // write_velocity_field_snapshot, 3D:2765-2786: '(3I6,6ES15.6)', k outer,
    // i fastest; x = (i-1)*xlen/nx and y = (j-1)*ylen/ny evaluated in that order.
    if (nx < 1 || ny < 1 || nz < 1 || !z || !u || !v || !w) return DNS3D_E_INVALID;
    File f(join(dir, numbered("velocity_field_", istep)), "w");
    if (!f.f) return DNS3D_E_IO;
    f.line("# DNS 3D Velocity Field Snapshot");
    f.line("# Time step: " + std::to_string(istep));
    f.line("# Time: " + fmt_f(time, 12, 6));
    f.line("# Columns: i, j, k, x, y, z, u, v, w");
    std::string buf;
    buf.reserve((size_t)nx * 126);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            buf.clear();
            const double y = (double)j * ylen / (double)ny;
            for (int i = 0; i < nx; ++i) {
                const size_t p = ((size_t)k * ny + j) * nx + i;
                const double x = (double)i * xlen / (double)nx;
                buf += fmt_i(i + 1, 6) + fmt_i(j + 1, 6) + fmt_i(k + 1, 6) + fmt_es(x, 15, 6) + fmt_es(y, 15, 6) +
                       fmt_es(z[k], 15, 6) + fmt_es(u[p], 15, 6) + fmt_es(v[p], 15, 6) + fmt_es(w[p], 15, 6) + "\n";
            }
            std::fputs(buf.c_str(), f.f);
        }
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_output_simulation_summary(const char* dir, const dns3d_config* c, const char* input_filename,
                                    const char* output_directory, const char* restart_filename, int restarted,
                                    int restart_step, double restart_time) {
    // write_simulation_summary, 3D:2594-2659; Start time is the local clock.
    if (!c) return DNS3D_E_INVALID;
    File f(join(dir, "simulation_summary.txt"), "w");
    if (!f.f) return DNS3D_E_IO;
    const std::time_t now = std::time(nullptr);
    std::tm tmv{};
    localtime_r(&now, &tmv);
    char ds[32], ts[32];
    std::snprintf(ds, sizeof ds, "%04d-%02d-%02d", tmv.tm_year + 1900, tmv.tm_mon + 1, tmv.tm_mday);
    std::snprintf(ts, sizeof ts, "%02d:%02d:%02d", tmv.tm_hour, tmv.tm_min, tmv.tm_sec);
    const std::string bar = "============================================";
    f.line(bar);
    f.line("   3D DNS SIMULATION SUMMARY");
    f.line(bar);
    f.line(" ");
    f.line(std::string(" Input file: ") + (input_filename ? input_filename : ""));
    f.line(std::string(" Output directory: ") + (output_directory ? output_directory : (dir ? dir : "")));
    f.line(std::string(" Start time: ") + ds);
    f.line(std::string("             ") + ts);
    f.line(" ");
    f.line(" GRID PARAMETERS:");
    f.line("   Grid size: " + std::to_string(c->nx) + " × " + std::to_string(c->ny) + " × " + std::to_string(c->nz));
    f.line("   Domain Lx: " + fmt_f(c->xlen, 8, 4));
    f.line("   Domain Ly: " + fmt_f(c->ylen, 8, 4));
    f.line("   Domain Lz: " + fmt_f(2.0, 8, 4));  // ybar = 2 (3D:742)
    f.line(" ");
    f.line(" SIMULATION PARAMETERS:");
    f.line("   Reynolds number: " + fmt_f(c->re, 10, 4));
    f.line("   Time step: " + fmt_f(c->dt, 10, 6));
    f.line("   Total steps: " + std::to_string(c->nsteps));
    f.line("   Output frequency: " + std::to_string(c->nwrt));
    f.line("   Total time: " + fmt_f((double)c->nsteps * c->dt, 10, 4));
    f.line(" ");
    f.line(" FLOW CONTROL:");
    f.line("   Method: " + std::to_string(c->flow_control_method));
    if (c->flow_control_method == 2) {
        f.line("   Target bulk velocity: " + fmt_f(c->target_bulk_velocity, 10, 6));
        f.line("   Controller gain: " + fmt_f(c->controller_gain, 10, 6));
        f.line("   Update frequency: " + std::to_string(c->controller_update_freq));
    }
    f.line(" ");
    f.line(" OUTPUT FILES:");
    f.line("   - simulation_summary.txt (this file)");
    f.line("   - output_time_series.dat (time evolution)");
    f.line("   - flow_statistics.dat (statistical summaries)");
    f.line("   - velocity_field_XXXXX.dat (field snapshots)");
    f.line("   - spanwise_profile_XXXXX.dat (averaged profiles)");
    f.line(" ");
    f.line(" RESTART CONFIGURATION (Phase 5):");
    f.line("   Restart write frequency: " + std::to_string(c->restart_write_freq));
    f.line(std::string("   Restart filename: ") + (restart_filename ? restart_filename : "restart.dat"));
    if (restarted) {
        f.line("   Restart mode: ENABLED (restarting from checkpoint)");
        f.line("   Restart step: " + std::to_string(restart_step));
        f.line("   Restart time: " + fmt_f(restart_time, 12, 6));
    } else {
        f.line("   Restart mode: DISABLED (new simulation)");
    }
    f.line(" ");
    f.line(bar);
    return f.close() ? DNS3D_OK : DNS3D_E_IO;
}

// Handle level, the reference's subroutine names.  Each reduces the device
// state for its numbers (dns3d_flow_statistics) at the handle's clock.

int dns3d_write_time_series_data(dns3d_handle* h, const char* dir) {
    dns3d_flow_stats st;
    int rc = dns3d_flow_statistics(h, &st, nullptr, nullptr, nullptr);
    if (rc && rc != DNS3D_E_NONFINITE) return rc;
    const int rw = dns3d_output_time_series_row(dir, &st);
    return rw ? rw : rc;
}

int dns3d_write_flow_statistics(dns3d_handle* h, const char* dir) {
    dns3d_flow_stats st;
    int rc = dns3d_flow_statistics(h, &st, nullptr, nullptr, nullptr);
    if (rc && rc != DNS3D_E_NONFINITE) return rc;
    const int rw = dns3d_output_flow_statistics(dir, &st);
    return rw ? rw : rc;
}

int dns3d_write_spanwise_averaged_profile(dns3d_handle* h, const char* dir) {
    dns3d_config c;
    int rc = dns3d_get_config(h, &c);
    if (rc) return rc;
    std::vector<double> prof(3 * (size_t)c.nz), z(c.nz), wz(c.nz);
    dns3d_flow_stats st;
    rc = dns3d_flow_statistics(h, &st, prof.data(), prof.data() + c.nz, prof.data() + 2 * c.nz);
    if (rc && rc != DNS3D_E_NONFINITE) return rc;
    const int rz = dns3d_lgl_nodes_weights(c.nz, z.data(), wz.data());
    if (rz) return rz;
    const int rw = dns3d_output_spanwise_profile(dir, st.step, st.time, c.nz, z.data(), prof.data(),
                                                 prof.data() + c.nz, prof.data() + 2 * c.nz);
    return rw ? rw : rc;
}

int dns3d_write_velocity_field_snapshot(dns3d_handle* h, const char* dir) {
    dns3d_config c;
    int rc = dns3d_get_config(h, &c);
    if (rc) return rc;
    int step = 0;
    double time = 0.0;
    if ((rc = dns3d_get_clock(h, &step, &time))) return rc;
    const size_t n = (size_t)c.nx * c.ny * c.nz;
    std::vector<double> u(n), v(n), w(n), z(c.nz), wz(c.nz);
    if ((rc = dns3d_get_state(h, u.data(), v.data(), w.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                              nullptr)))
        return rc;
    if ((rc = dns3d_lgl_nodes_weights(c.nz, z.data(), wz.data()))) return rc;
    return dns3d_output_velocity_snapshot(dir, step, time, c.nx, c.ny, c.nz, c.xlen, c.ylen, z.data(), u.data(),
                                          v.data(), w.data());
}

}  // extern "C"

// Restart files in the reference's stream format (write_restart_file_3d and
// read_restart_file_3d, DNS_pressure_BC_3D.f90:2976-3209), over the public
// C-ABI.  The layout is fixed by the reference so that files move between the
// Fortran program and this library in both directions.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dns3d_capi.h"

namespace {

const char kTag[] = "DNS3D_RESTART_v1.0";  // 18 characters, no terminator in the file
constexpr double kPi = 3.14159265358979323846;

struct File {
    std::FILE* f = nullptr;
    explicit File(std::FILE* p) : f(p) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

bool put(std::FILE* f, const void* p, size_t n) { return std::fwrite(p, 1, n, f) == n; }
bool get(std::FILE* f, void* p, size_t n) { return std::fread(p, 1, n, f) == n; }

bool put_field(std::FILE* f, const double* a, size_t n) {
    if (a) return put(f, a, n * sizeof(double));
    std::vector<double> z(n, 0.0);
    return put(f, z.data(), n * sizeof(double));
}
bool get_field(std::FILE* f, double* a, size_t n) {
    if (a) return get(f, a, n * sizeof(double));
    return std::fseek(f, (long)(n * sizeof(double)), SEEK_CUR) == 0;
}

}  // namespace

extern "C" {

int dns3d_restart_write(const char* path, const dns3d_restart_header* hdr, const double* u, const double* v,
                        const double* w, const double* un, const double* vn, const double* wn,
                        const double* p_total, const dns3d_pi_state* pi) {
    if (!path || !hdr || hdr->nx < 1 || hdr->ny < 1 || hdr->nz < 1) return DNS3D_E_INVALID;
    File fh(std::fopen(path, "wb"));
    if (!fh.f) return DNS3D_E_IO;
    const size_t n = (size_t)hdr->nx * hdr->ny * hdr->nz;
    const int istep = hdr->istep;
    const int dims[3] = {hdr->nx, hdr->ny, hdr->nz};
    const double td[2] = {hdr->time, hdr->dt};
    const double rab[3] = {hdr->re, hdr->alpha, hdr->beta};
    const double pis[4] = {pi ? pi->current_pressure_gradient : 0.0, pi ? pi->current_bulk_velocity : 0.0,
                           pi ? pi->bulk_velocity_error_integral : 0.0, pi ? pi->bulk_velocity_error_prev : 0.0};
    bool ok = put(fh.f, kTag, 18) && put(fh.f, &istep, 4) && put(fh.f, td, 16) && put(fh.f, dims, 12) &&
              put(fh.f, rab, 24);
    const double* fields[7] = {u, v, w, un, vn, wn, p_total};
    for (int k = 0; k < 7 && ok; ++k) ok = put_field(fh.f, fields[k], n);
    ok = ok && put(fh.f, pis, 32);
    return ok ? DNS3D_OK : DNS3D_E_IO;
}

int dns3d_restart_read(const char* path, dns3d_restart_header* hdr, double* u, double* v, double* w,
                       double* un, double* vn, double* wn, double* p_total, dns3d_pi_state* pi) {
    if (!path || !hdr) return DNS3D_E_INVALID;
    File fh(std::fopen(path, "rb"));
    if (!fh.f) return DNS3D_E_IO;
    char tag[18];
    if (!get(fh.f, tag, 18) || std::memcmp(tag, kTag, 18) != 0) return DNS3D_E_IO;
    int istep = 0, dims[3] = {0, 0, 0};
    double td[2], rab[3];
    if (!get(fh.f, &istep, 4) || !get(fh.f, td, 16) || !get(fh.f, dims, 12)) return DNS3D_E_IO;
    if (dims[0] != hdr->nx || dims[1] != hdr->ny || dims[2] != hdr->nz) return DNS3D_E_INVALID;
    if (!get(fh.f, rab, 24)) return DNS3D_E_IO;
    hdr->istep = istep;
    hdr->time = td[0];
    hdr->dt = td[1];
    hdr->re = rab[0];
    hdr->alpha = rab[1];
    hdr->beta = rab[2];
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    double* fields[7] = {u, v, w, un, vn, wn, p_total};
    for (int k = 0; k < 7; ++k)
        if (!get_field(fh.f, fields[k], n)) return DNS3D_E_IO;
    double pis[4];
    if (get(fh.f, pis, 32) && pi) {  // a short file keeps the defaults (3D:3187-3193)
        pi->current_pressure_gradient = pis[0];
        pi->current_bulk_velocity = pis[1];
        pi->bulk_velocity_error_integral = pis[2];
        pi->bulk_velocity_error_prev = pis[3];
    }
    return DNS3D_OK;
}

int dns3d_save_restart(dns3d_handle* h, const char* path, int istep, double time) {
    if (!h || !path) return DNS3D_E_INVALID;
    dns3d_config c;
    int rc = dns3d_get_config(h, &c);
    if (rc) return rc;
    const size_t n = (size_t)c.nx * c.ny * c.nz;
    std::vector<double> u(n), v(n), w(n), p(n);
    dns3d_pi_state pi;
    rc = dns3d_get_state(h, u.data(), v.data(), w.data(), p.data(), nullptr, nullptr, nullptr, nullptr, &pi);
    if (rc) return rc;
    dns3d_restart_header hdr{};
    hdr.istep = istep;
    hdr.nx = c.nx;
    hdr.ny = c.ny;
    hdr.nz = c.nz;
    hdr.time = time;
    hdr.dt = c.dt;
    hdr.re = c.re;
    hdr.alpha = 2.0 * kPi / c.xlen;  // setup_grid_3d overrides the namelist alpha, beta (3D:740-741)
    hdr.beta = 2.0 * kPi / c.ylen;
    return dns3d_restart_write(path, &hdr, u.data(), v.data(), w.data(), u.data(), v.data(), w.data(), p.data(),
                               &pi);
}

int dns3d_load_restart(dns3d_handle* h, const char* path, int* istep, double* time) {
    if (!h || !path) return DNS3D_E_INVALID;
    dns3d_config c;
    int rc = dns3d_get_config(h, &c);
    if (rc) return rc;
    const size_t n = (size_t)c.nx * c.ny * c.nz;
    std::vector<double> u(n), v(n), w(n), p(n);
    dns3d_pi_state pi;
    rc = dns3d_get_state(h, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &pi);
    if (rc) return rc;
    // defaults of read_input_3d for the scalars a short file lacks (3D:623-635)
    pi.current_pressure_gradient = c.target_pressure_gradient;
    pi.current_bulk_velocity = 0.0;
    pi.bulk_velocity_error_integral = 0.0;
    pi.bulk_velocity_error_prev = 0.0;
    dns3d_restart_header hdr{};
    hdr.nx = c.nx;
    hdr.ny = c.ny;
    hdr.nz = c.nz;
    rc = dns3d_restart_read(path, &hdr, u.data(), v.data(), w.data(), nullptr, nullptr, nullptr, p.data(), &pi);
    if (rc) return rc;
    std::vector<double> zero((size_t)c.nx * c.ny, 0.0);
    rc = dns3d_set_state(h, u.data(), v.data(), w.data(), p.data(), zero.data(), zero.data(), zero.data(),
                         zero.data(), &pi);
    if (rc) return rc;
    if (istep) *istep = hdr.istep;
    if (time) *time = hdr.time;
    return dns3d_set_clock(h, hdr.istep, hdr.time);
}

}  // extern "C"

// Host-side setup restated from the reference: LGL nodes, weights and
// differentiation matrix (lgl_module.f90), and the namelist reader of
// read_input_3d (DNS_pressure_BC_3D.f90:554-708).
//
// Built with -ffp-contract=off so that the operators are the same on every
// host architecture (no fused multiply-add contraction in the recurrences).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "dns3d_internal.cuh"

namespace dns3d {

namespace {

// legendre_poly (lgl_module.f90:86-110)
double legendre(int n, double x) {
    if (n == 0) return 1.0;
    if (n == 1) return x;
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; ++k) {
        const double p2 = ((double)(2 * k - 1) * x * p1 - (double)(k - 1) * p0) / (double)k;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// legendre_poly_and_deriv (lgl_module.f90:115-155)
void legendre_d(int n, double x, double& p, double& dp, double& d2p) {
    if (n == 0) { p = 1.0; dp = 0.0; d2p = 0.0; return; }
    if (n == 1) { p = x; dp = 1.0; d2p = 0.0; return; }
    double p0 = 1.0, dp0 = 0.0, d2p0 = 0.0;
    double p1 = x, dp1 = 1.0, d2p1 = 0.0;
    for (int k = 2; k <= n; ++k) {
        const double a = (double)(2 * k - 1), b = (double)(k - 1), c = (double)k;
        const double p2 = (a * x * p1 - b * p0) / c;
        const double dp2 = (a * (x * dp1 + p1) - b * dp0) / c;
        const double d2p2 = (a * (x * d2p1 + 2.0 * dp1) - b * d2p0) / c;
        p0 = p1; p1 = p2;
        dp0 = dp1; dp1 = dp2;
        d2p0 = d2p1; d2p1 = d2p2;
    }
    p = p1; dp = dp1; d2p = d2p1;
}

}  // namespace

// lgl_nodes_weights (lgl_module.f90:30-80): Newton on P'_{n-1} from the
// Chebyshev guesses -cos(pi (i-1)/(n-1)), |dx| < 1e-15 or 100 iterations.
void lgl_nodes_weights(int n, std::vector<double>& x, std::vector<double>& w) {
    const double pi = 3.14159265358979323846;
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    if (n == 1) { x[0] = 0.0; w[0] = 2.0; return; }
    if (n == 2) { x[0] = -1.0; x[1] = 1.0; w[0] = w[1] = 1.0; return; }
    x[0] = -1.0;
    x[n - 1] = 1.0;
    w[0] = 2.0 / (double)(n * (n - 1));
    w[n - 1] = w[0];
    for (int i = 2; i <= n - 1; ++i) {
        double xi = -std::cos(pi * (double)(i - 1) / (double)(n - 1));
        for (int it = 0; it < 100; ++it) {
            const double xo = xi;
            double p, dp, d2p;
            legendre_d(n - 1, xi, p, dp, d2p);
            xi = xo - dp / d2p;
            if (std::fabs(xi - xo) < 1.0e-15) break;
        }
        x[i - 1] = xi;
        const double p = legendre(n - 1, xi);
        w[i - 1] = 2.0 / ((double)(n * (n - 1)) * p * p);
    }
}

// differentiation_matrix (lgl_module.f90:211-263), row-major d[i*n+j].
// guard = true keeps the reference's "|prod2| > 1e-15 else 0" rule.
void lgl_diff_matrix(const std::vector<double>& x, bool guard, std::vector<double>& d) {
    const int n = (int)x.size();
    d.assign((size_t)n * n, 0.0);
    if (n == 1) return;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (i == j) {
                double s = 0.0;
                for (int k = 0; k < n; ++k)
                    if (k != i) s += 1.0 / (x[i] - x[k]);
                d[(size_t)i * n + i] = s;
            } else {
                double p1 = 1.0, p2 = 1.0;
                for (int k = 0; k < n; ++k) {
                    if (k != i && k != j) p1 *= x[i] - x[k];
                    if (k != j) p2 *= x[j] - x[k];
                }
                d[(size_t)i * n + j] = (std::fabs(p2) > 1.0e-15 || !guard) ? p1 / p2 : 0.0;
            }
        }
    }
}

// Cyclic Jacobi rotations until the off-diagonal mass is at rounding level.
void jacobi_eigen(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& y) {
    y.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) y[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double& { return a[(size_t)i * n + j]; };
    double diag2 = 0.0;
    for (int i = 0; i < n; ++i) diag2 += A(i, i) * A(i, i);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += A(p, q) * A(p, q);
        if (off <= 1e-32 * diag2) break;
        for (int p = 0; p < n; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (std::fabs(apq) < 1e-300) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double ykp = y[(size_t)k * n + p], ykq = y[(size_t)k * n + q];
                    y[(size_t)k * n + p] = c * ykp - s * ykq;
                    y[(size_t)k * n + q] = s * ykp + c * ykq;
                }
            }
        }
    }
    // sort ascending
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int i, int j) { return A(i, i) < A(j, j); });
    w.resize(n);
    std::vector<double> ys((size_t)n * n);
    for (int c = 0; c < n; ++c) {
        w[c] = A(idx[c], idx[c]);
        for (int r = 0; r < n; ++r) ys[(size_t)r * n + c] = y[(size_t)r * n + idx[c]];
    }
    y.swap(ys);
}

// ------------------------------------------------------------------ namelist
namespace {

std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}
std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

bool parse_real(const std::string& v, double& out) {
    std::string t = v;
    for (auto& c : t)
        if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    out = std::strtod(t.c_str(), &end);
    return end && end != t.c_str() && trim(end).empty();
}
bool parse_int(const std::string& v, int& out) {
    char* end = nullptr;
    long x = std::strtol(v.c_str(), &end, 10);
    if (!end || end == v.c_str() || !trim(end).empty()) return false;
    out = (int)x;
    return true;
}
bool parse_int64(const std::string& v, long long& out) {
    char* end = nullptr;
    long long x = std::strtoll(v.c_str(), &end, 10);
    if (!end || end == v.c_str() || !trim(end).empty()) return false;
    out = x;
    return true;
}
bool parse_logical(const std::string& v, int& out) {
    std::string t = lower(trim(v));
    if (!t.empty() && t[0] == '.') t = t.substr(1);
    if (t.empty()) return false;
    if (t[0] == 't') { out = 1; return true; }
    if (t[0] == 'f') { out = 0; return true; }
    return false;
}

bool assign(dns3d_config* c, const std::string& group, const std::string& key, const std::string& val) {
    int i;
    double r;
#define INT_KEY(name, field) if (key == name) { if (!parse_int(val, i)) return false; c->field = i; return true; }
#define REAL_KEY(name, field) if (key == name) { if (!parse_real(val, r)) return false; c->field = r; return true; }
#define LOG_KEY(name, field) if (key == name) { if (!parse_logical(val, i)) return false; c->field = i; return true; }
    if (group == "grid") {
        INT_KEY("nx_input", nx) INT_KEY("ny_input", ny) INT_KEY("nz_input", nz)
    } else if (group == "time_control") {
        INT_KEY("istart", istart) REAL_KEY("dt", dt) INT_KEY("nsteps", nsteps) INT_KEY("nwrt", nwrt)
        INT_KEY("restart_write_freq", restart_write_freq)
    } else if (group == "simulation") {
        REAL_KEY("re", re) REAL_KEY("xlen", xlen) REAL_KEY("ylen", ylen)
        REAL_KEY("u_centerline", u_centerline) LOG_KEY("use_crank_nicolson", use_crank_nicolson)
        REAL_KEY("cgstol", cgstol)
    } else if (group == "flow_control") {
        INT_KEY("flow_control_method", flow_control_method)
        REAL_KEY("target_pressure_gradient", target_pressure_gradient)
        REAL_KEY("target_bulk_velocity", target_bulk_velocity) REAL_KEY("controller_gain", controller_gain)
        INT_KEY("controller_update_freq", controller_update_freq)
    } else if (group == "perturbations") {
        LOG_KEY("enable_perturbations", enable_perturbations)
        REAL_KEY("perturbation_amplitude", perturbation_amplitude)
        LOG_KEY("zero_w_perturbations", zero_w_perturbations)
        LOG_KEY("use_analytical_perturbations", use_analytical_perturbations)
        INT_KEY("analytical_mode_x", analytical_mode_x) INT_KEY("analytical_mode_y", analytical_mode_y)
        // extension keys of this library: white-noise amplitude, perturbation seed
        REAL_KEY("noise_amplitude", noise_amplitude)
        if (key == "perturbation_seed") {
            long long s64;
            if (!parse_int64(val, s64)) return false;
            c->perturbation_seed = s64;
            return true;
        }
    } else if (group == "pressure_solver") {
        LOG_KEY("use_weak_form_divergence", use_weak_form_divergence)
    } else if (group == "computational") {
        LOG_KEY("use_dealias_23_rule", use_dealias_23_rule)
        // extension keys of this library (not read by the reference)
        LOG_KEY("lgl_dmatrix_guard", lgl_dmatrix_guard)
        INT_KEY("convection_scheme", convection_scheme) INT_KEY("linear_solver", linear_solver)
        LOG_KEY("poisson_refinement", poisson_refinement)
    }
#undef INT_KEY
#undef REAL_KEY
#undef LOG_KEY
    return true;  // keys the step does not use (alpha, beta, ta, ybar, cs, ...) are accepted
}

}  // namespace

int read_namelist_file(const char* path, dns3d_config* cfg) {
    std::ifstream in(path);
    if (!in) return DNS3D_E_IO;
    std::stringstream ss;
    ss << in.rdbuf();
    std::string text = ss.str();
    // strip comments ('!' to end of line) outside quotes
    std::string clean;
    bool q = false;
    for (size_t i = 0; i < text.size(); ++i) {
        const char ch = text[i];
        if (ch == '\'' || ch == '"') q = !q;
        if (ch == '!' && !q) {
            while (i < text.size() && text[i] != '\n') ++i;
            clean.push_back('\n');
            continue;
        }
        clean.push_back(ch);
    }
    size_t pos = 0;
    while (true) {
        const size_t amp = clean.find('&', pos);
        if (amp == std::string::npos) break;
        size_t e = amp + 1;
        while (e < clean.size() && (std::isalnum((unsigned char)clean[e]) || clean[e] == '_')) ++e;
        const std::string group = lower(clean.substr(amp + 1, e - amp - 1));
        size_t end = clean.find('/', e);
        if (end == std::string::npos) return DNS3D_E_IO;
        const std::string body = clean.substr(e, end - e);
        // split "key = value" pairs separated by commas or newlines
        size_t p = 0;
        while (p < body.size()) {
            const size_t eq = body.find('=', p);
            if (eq == std::string::npos) break;
            std::string key = lower(trim(body.substr(p, eq - p)));
            const size_t ks = key.find_last_of(" \t\r\n,");
            if (ks != std::string::npos) key = key.substr(ks + 1);
            size_t vend = eq + 1;
            // value runs to the next comma/newline not inside quotes
            bool inq = false;
            while (vend < body.size()) {
                const char ch = body[vend];
                if (ch == '\'' || ch == '"') inq = !inq;
                if (!inq && (ch == ',' || ch == '\n')) break;
                ++vend;
            }
            const std::string val = trim(body.substr(eq + 1, vend - eq - 1));
            if (!key.empty() && !assign(cfg, group, key, val)) return DNS3D_E_IO;
            p = vend + 1;
        }
        pos = end + 1;
    }
    return DNS3D_OK;
}

}  // namespace dns3d

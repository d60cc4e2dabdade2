// waveinput.dat reader and host-side spectral helpers.
//
// The grammar, keyword prefixes, defaults and quirks follow the reference's
// wave_Initialize (CFDwavemaker.cpp:2065-2149) and process_inputdata
// (CFDwavemaker.cpp:232-1530): '#' starts a comment, the first line carries
// "@vNNN" with NNN >= 300, sections are "[...]" headers, keywords are matched
// by prefix, irregular components are stable-sorted by omega, and the
// amplitudes are normalised/amplified after parsing (Irregular.cpp:1282).
// Instead of calling exit() on bad input, errors are returned as E_PARSE.
#include "cfdwm.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>

namespace cfdwm {
namespace {

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

bool starts(const std::string &s, const char *p) { return s.compare(0, std::strlen(p), p) == 0; }

std::vector<std::string> tokens(const std::string &s) {
    std::istringstream is(s);
    std::vector<std::string> t;
    std::string w;
    while (is >> w) t.push_back(w);
    return t;
}

// operator>> into a double: a failed extraction yields 0.
double num(const std::vector<std::string> &t, size_t i) {
    if (i >= t.size()) return 0.0;
    char *end = nullptr;
    double v = std::strtod(t[i].c_str(), &end);
    return (end == t[i].c_str()) ? 0.0 : v;
}
int inum(const std::vector<std::string> &t, size_t i) {
    if (i >= t.size()) return 0;
    return std::atoi(t[i].c_str());
}

// std::getline over the comment-stripped text, with eof() semantics of
// std::istringstream (the read after the last line sets eof and yields "").
struct Lines {
    std::vector<std::string> v;
    size_t pos = 0;
    bool eof = false;
    explicit Lines(const std::string &text) {
        std::string cur;
        for (char ch : text) {
            if (ch == '\n') { v.push_back(cur); cur.clear(); }
            else cur.push_back(ch);
        }
        if (!cur.empty()) v.push_back(cur);
    }
    std::string get() {
        if (pos >= v.size()) { eof = true; return std::string(); }
        return v[pos++];
    }
};

int fail(Config &cfg, const std::string &msg) {
    cfg.error = msg;
    return E_PARSE;
}

}  // namespace

int parse_waveinput_text(const std::string &raw, Config &cfg) {
    // comment stripping and the version line (CFDwavemaker.cpp:2113-2138)
    std::string res;
    {
        std::istringstream is(raw);
        std::string line;
        while (std::getline(is, line)) {
            size_t h = line.find('#');
            if (h != std::string::npos) line.erase(h);
            if (!line.empty()) res += line + "\n";
        }
    }
    {
        std::string first = trim(res.substr(0, res.find('\n')));
        if (first.compare(0, 2, "@v") != 0) return fail(cfg, "missing @vNNN version line");
        if (std::atoi(first.substr(2, 3).c_str()) < 300) return fail(cfg, "input file version < 300");
    }
    Lines f(res);
    bool skip = false;
    std::string line;
    while (!f.eof) {
        if (skip) skip = false;
        else line = trim(f.get());

        if (line == "[wave type]") {
            line = trim(f.get());
            if (line == "irregular" || line == "1") cfg.wavetype = WT_IRREGULAR;
            else if (line == "piston") cfg.wavetype = WT_PISTON;
            else if (line == "regular") cfg.wavetype = WT_REGULAR;
            else if (line == "swd") cfg.wavetype = WT_SWD;
            else if (line == "vtk") cfg.wavetype = WT_VTK;
            else if (line == "slope") cfg.wavetype = WT_SLOPE;
            else return fail(cfg, "unknown wave type: " + line);
        }
        if (line == "[general input data]") {
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "depth")) cfg.depth = num(t, 1);
                if (starts(line, "mtheta")) cfg.mtheta = num(t, 1);
                if (starts(line, "normalize")) cfg.normalize = inum(t, 1) != 0;
                if (starts(line, "amplify")) cfg.ampl = num(t, 1);
                if (starts(line, "swl")) cfg.swl = num(t, 1);
                if (starts(line, "gravity")) cfg.gravity = num(t, 1);
                if (starts(line, "rho")) cfg.rho = num(t, 1);
                if (starts(line, "nhpres_include_kinetic"))
                    cfg.nhpres_kinetic = t.size() > 1 && starts(t[1], "true");
                if (starts(line, "[")) { skip = true; break; }
            }
        }
        if (line == "[wave reference point]") {
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "time")) cfg.tofmax = num(t, 1);
                if (starts(line, "x")) cfg.x_pos = num(t, 1);
                if (starts(line, "y")) cfg.y_pos = num(t, 1);
                if (starts(line, "[")) { skip = true; break; }
            }
        }
        if (line == "[ramps]") {
            static const char *names[6] = {"time_rampup", "time_rampdown", "x_rampup",
                                           "x_rampdown", "y_rampup", "y_rampdown"};
            cfg.ramp.init = true;
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                for (int q = 0; q < 6; q++)
                    if (starts(line, names[q])) {
                        cfg.ramp.flags |= 1 << q;
                        cfg.ramp.lim[2 * q] = num(t, 1);
                        cfg.ramp.lim[2 * q + 1] = num(t, 2);
                    }
                if (starts(line, "[")) { skip = true; break; }
            }
        }
        if (line == "[wave input irregular]") {
            if (cfg.wavetype != WT_IRREGULAR)
                return fail(cfg, "irregular wave components do not match the wave type");
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "kinematics_surf_extrap")) {
                    cfg.extrapolation_met = inum(t, 1);
                    if (cfg.extrapolation_met == 2) cfg.order = 2;
                    else if (cfg.extrapolation_met == 1 || cfg.extrapolation_met == 0) cfg.order = 0;
                    else return fail(cfg, "unknown extrapolation method");
                }
                if (starts(line, "cutoff")) cfg.dw_cutoff = num(t, 1);
                if (starts(line, "bandwidth")) {
                    std::string v = t.size() > 1 ? t[1] : std::string();
                    if (starts(v, "off")) {
                    } else if (starts(v, "auto")) cfg.bw_auto = true;
                    else cfg.dw_bandwidth = std::atof(v.c_str());
                }
                if (starts(line, "individual_ramp") && t.size() > 1 && starts(t[1], "true"))
                    cfg.individual_ramp = true;
                if (starts(line, "vertical_theory"))
                    cfg.vertical_theory = (t.size() > 1 && starts(t[1], "smit")) ? 1 : 0;
                if (starts(line, "nfreq")) break;
            }
            if (!starts(line, "nfreq")) return fail(cfg, "parameter nfreq missing");
            cfg.nfreq = inum(tokens(line), 1);
            line = trim(f.get());
            if (!starts(line, "ndir")) return fail(cfg, "parameter ndir missing");
            cfg.ndir = inum(tokens(line), 1);
            std::vector<double> om, A, k, ph, th, rt, st, du;
            if (cfg.ndir == 0) {
                cfg.ndir = 1;
                for (int i = 0; i < cfg.nfreq; i++) {
                    std::string r = f.get();
                    if (starts(r, "[")) return fail(cfg, "not enough frequency components");
                    auto t = tokens(r);
                    om.push_back(num(t, 0)); A.push_back(num(t, 1)); k.push_back(num(t, 2));
                    ph.push_back(num(t, 3)); th.push_back(num(t, 4));
                    if (cfg.individual_ramp) {
                        rt.push_back(num(t, 5)); st.push_back(num(t, 6)); du.push_back(num(t, 7));
                    } else {
                        rt.push_back(0.0); st.push_back(-SMALL); du.push_back(HUGE_);
                    }
                }
            } else {
                std::vector<double> fo, fa, fk, fp, dth, dd;
                for (int i = 0; i < cfg.nfreq; i++) {
                    auto t = tokens(f.get());
                    fo.push_back(num(t, 0)); fa.push_back(num(t, 1)); fk.push_back(num(t, 2));
                    fp.push_back(num(t, 3));
                }
                for (int j = 0; j < cfg.ndir; j++) {
                    std::string r = f.get();
                    if (starts(r, "[")) return fail(cfg, "too few directional components");
                    auto t = tokens(r);
                    dth.push_back(num(t, 0)); dd.push_back(num(t, 1));
                }
                for (int i = 0; i < cfg.nfreq; i++)
                    for (int j = 0; j < cfg.ndir; j++) {
                        om.push_back(fo[i]); k.push_back(fk[i]); A.push_back(fa[i] * dd[j]);
                        ph.push_back(fp[i]); th.push_back(dth[j]);
                        rt.push_back(0.0); st.push_back(-SMALL); du.push_back(HUGE_);
                    }
            }
            std::vector<size_t> idx(om.size());
            std::iota(idx.begin(), idx.end(), 0);
            std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return om[a] < om[b]; });
            for (size_t i : idx) {
                cfg.omega.push_back(om[i]); cfg.A.push_back(A[i]); cfg.k.push_back(k[i]);
                cfg.phase.push_back(ph[i]); cfg.theta.push_back(th[i]);
                cfg.ramptime.push_back(rt[i]); cfg.starttime.push_back(st[i]);
                cfg.duration.push_back(du[i]);
            }
            cfg.property_read = true;
        }
        if (line == "[lsgrid2vtk]") {
            // .vtu output of the s-grid (CFDwavemaker.cpp:1205-1245); the
            // [lsgrid] section must come first
            if (cfg.wavetype != WT_IRR_SGRID)
                return fail(cfg, "VTK output only works in combination with LSgrid");
            LsgridCfg &g = cfg.lsgrid;
            g.dump_vtk = true;
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "storage_path") && t.size() > 1) g.vtk_path = t[1];
                if (starts(line, "filename") && t.size() > 1) g.vtk_prefix = t[1];
                if (starts(line, "vtk_timelabel") && t.size() > 1) g.vtk_timelabel = t[1];
                if (starts(line, "[")) { skip = true; break; }
            }
        }
        if (line == "[wave input piston]" || line == "[sloping water]" ||
            line == "[wave input swd]" || line == "[wave input vtk]") {
            // Recognised sections of paths this build does not serve; their
            // keywords are consumed so that parsing continues.
            while (!f.eof) {
                line = trim(f.get());
                if (starts(line, "[")) { skip = true; break; }
            }
        }
        if (line == "[wave input regular]") {
            if (cfg.wavetype != WT_REGULAR)
                return fail(cfg, "regular wave properties do not match the wave type");
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "theory_type")) {
                    std::string tt = t.size() > 1 ? t[1] : std::string();
                    cfg.regular_theory = (tt == "stream" || tt == "fenton") ? 1 : 0;
                }
                if (starts(line, "wave_order")) cfg.wave_order = inum(t, 1);
                if (starts(line, "wave_length")) {
                    cfg.wave_length = num(t, 1);
                    cfg.regular_specify_length = true;
                    cfg.wave_period = period_from_length(cfg.wave_length, cfg.depth, cfg.gravity);
                }
                if (starts(line, "wave_period")) {
                    cfg.wave_period = num(t, 1);
                    cfg.regular_specify_length = false;
                    cfg.wave_length = wavelength_from_period(cfg.wave_period, cfg.depth, cfg.gravity);
                }
                if (starts(line, "wave_height")) cfg.wave_height = num(t, 1);
                if (starts(line, "current_speed")) cfg.current = num(t, 1);
                if (starts(line, "[")) { skip = true; break; }
            }
            cfg.property_read = true;
        }
        if (line == "[lsgrid]") {
            LsgridCfg &g = cfg.lsgrid;
            g.present = true;
            while (!f.eof) {
                line = trim(f.get());
                auto t = tokens(line);
                if (starts(line, "bounds")) for (int q = 0; q < 4; q++) g.domain[q] = num(t, 1 + q);
                if (starts(line, "nx")) g.nx = inum(t, 1);
                if (starts(line, "ny")) g.ny = inum(t, 1);
                if (starts(line, "nl")) g.nl = inum(t, 1);
                if (starts(line, "t0")) g.t0 = num(t, 1);
                if (starts(line, "dt")) g.dt = num(t, 1);
                if (starts(line, "stretch_params")) { g.tan_a = num(t, 1); g.tan_b = num(t, 2); }
                if (starts(line, "ignore_subdomain")) {
                    for (int q = 0; q < 4; q++) g.domain_ignore[q] = num(t, 1 + q);
                    g.ignore_domain = true;
                }
                if (starts(line, "ignore_at_init")) g.ignore_at_init = inum(t, 1) != 0;
                if (starts(line, "init_only")) g.init_only = inum(t, 1) != 0;
                if (starts(line, "[")) { skip = true; break; }
            }
            if (cfg.wavetype == WT_IRREGULAR) cfg.wavetype = WT_IRR_SGRID;
            else if (cfg.wavetype == WT_SWD) cfg.wavetype = WT_SWD_SGRID;
            else return fail(cfg, "the s-grid needs irregular second order theory or swd");
        }
    }
    if (cfg.wavetype == WT_IRR_SGRID && cfg.order != 2)
        return fail(cfg, "the s-grid uses second order theory (kinematics_surf_extrap 2)");
    if (cfg.wavetype == WT_IRREGULAR || cfg.wavetype == WT_IRR_SGRID) {
        if (!cfg.property_read) return fail(cfg, "irregular wave selected but no components given");
        if (cfg.bw_auto) {
            // Irregular::bandwidth_estimator (Irregular.cpp:1439-1452), before normalisation
            if (cfg.ndir > 1) return fail(cfg, "automatic bandwidth needs a single direction");
            double m[3];
            spectral_moments(cfg, m);
            cfg.dw_bandwidth = 0.7 * (m[1] / m[0]);
        }
        // Irregular::normalize_data (Irregular.cpp:1282-1297)
        double sumA = 0.0;
        for (double a : cfg.A) sumA += a;
        for (size_t i = 0; i < cfg.A.size(); i++) {
            if (cfg.normalize) { cfg.A[i] = cfg.ampl * cfg.A[i] / sumA; cfg.phase[i] = 0.0; }
            else cfg.A[i] = cfg.ampl * cfg.A[i];
        }
    }
    if (cfg.wavetype == WT_REGULAR && !cfg.property_read)
        return fail(cfg, "regular wave selected but no wave properties given");
    return OK;
}

int read_waveinput_file(std::string &text, std::string &where) {
    static const char *paths[4] = {"./waveinput.dat", "./constant/waveinput.dat",
                                   "../input_files/waveinput.dat", "../waveinput.dat"};
    for (const char *p : paths) {
        std::ifstream fid(p);
        if (!fid.fail()) {
            std::stringstream ss;
            ss << fid.rdbuf();
            text = ss.str();
            where = p;
            return OK;
        }
    }
    return E_NO_FILE;
}

// Irregular::spectral_moments (Irregular.cpp:1336-1369): nfreq-1 terms.
void spectral_moments(const Config &c, double m[3]) {
    m[0] = m[1] = m[2] = 0.0;
    for (int i = 0; i < c.nfreq - 1; i++) {
        m[0] += c.A[i] * c.A[i] / 2.;
        m[1] += c.omega[i] * c.A[i] * c.A[i] / 2.;
        m[2] += c.omega[i] * c.omega[i] * c.A[i] * c.A[i] / 2.;
    }
}

// Irregular::interpolate with extrapolation (Irregular.cpp:1311-1334).
static double interp(const std::vector<double> &xd, const std::vector<double> &yd, double x) {
    int size = (int)xd.size(), i = 0;
    if (size < 2) return size ? yd[0] : 0.0;
    if (x >= xd[size - 2]) i = size - 2;
    else while (x > xd[i + 1]) i++;
    double xL = xd[i], yL = yd[i], xR = xd[i + 1], yR = yd[i + 1];
    return yL + (yR - yL) / (xR - xL) * (x - xL);
}

double phase_speed(const Config &c, int opt) {
    double m[3];
    spectral_moments(c, m);
    double t1 = 2. * PI_FULL * (m[0] / m[1]), t2 = 2. * PI_FULL * std::sqrt(m[0] / m[2]);
    double w1 = 2 * PI_FULL / t1, w2 = 2 * PI_FULL / t2;
    if (opt == 1) return w1 / interp(c.omega, c.k, w1);
    if (opt == 2) return w2 / interp(c.omega, c.k, w2);
    return 0.;
}
double mean_wave_length(const Config &c, int opt) {
    double m[3];
    spectral_moments(c, m);
    double t1 = 2. * PI_FULL * (m[0] / m[1]), t2 = 2. * PI_FULL * std::sqrt(m[0] / m[2]);
    double w1 = 2 * PI_FULL / t1, w2 = 2 * PI_FULL / t2;
    if (opt == 1) return (2. * PI_FULL) / interp(c.omega, c.k, w1);
    if (opt == 2) return (2. * PI_FULL) / interp(c.omega, c.k, w2);
    return 0.;
}
double mean_wave_period(const Config &c, int opt) {
    double m[3];
    spectral_moments(c, m);
    if (opt == 1) return 2. * PI_FULL * (m[0] / m[1]);
    if (opt == 2) return 2. * PI_FULL * std::sqrt(m[0] / m[2]);
    return 0.;
}

// Linear dispersion, Stokes5.cpp:187-229.
double wavenumber_from_period(double T, double depth, double g) {
    if (T <= 0.0 || depth <= 0.0 || g <= 0.0) return 0.0;
    const double omega = 2.0 * PI_FULL / T;
    double kk = 0.5 * (omega * omega / g + omega / std::sqrt(g * depth));
    for (int it = 0; it < 40; ++it) {
        double th = std::tanh(kk * depth);
        double f = g * kk * th - omega * omega;
        if (std::fabs(f) < 1e-14) break;
        double df = g * (th + kk * depth * (1.0 - th * th));
        if (std::fabs(df) < 1e-14) break;
        double dk = -f / df;
        kk += dk;
        if (kk < 1e-12) kk = 1e-12;
        if (std::fabs(dk) < 1e-12 * kk) break;
    }
    return kk;
}
double wavelength_from_period(double T, double depth, double g) {
    double kk = wavenumber_from_period(T, depth, g);
    return (kk > 0.0) ? 2.0 * PI_FULL / kk : 0.0;
}
double period_from_length(double L, double depth, double g) {
    if (L <= 0.0 || depth <= 0.0 || g <= 0.0) return 0.0;
    double kk = 2.0 * PI_FULL / L;
    return 2.0 * PI_FULL / std::sqrt(g * kk * std::tanh(kk * depth));
}

// Irregular::dumpSpectralComponents (Irregular.cpp:1456-1468): the reference
// writes ./spectral_components.dat on every irregular initialisation.
void dump_spectral_components(const Config &c) {
    FILE *fp = std::fopen("./spectral_components.dat", "w");
    if (!fp) return;
    std::fprintf(fp, "# spectral wave data output\n# [irregular wave components]\n");
    std::fprintf(fp, "# nfreq %d\n# ndir 0\n", c.nfreq);
    std::fprintf(fp, "# omega [rad/s]    a[m]       k[rad/m]        phi[rad]    theta[rad]\n");
    for (int i = 0; i < c.nfreq && i < (int)c.omega.size(); i++)
        std::fprintf(fp, "%12.5E  %12.5E  %12.5E  %12.5E  %12.5E\n", c.omega[i], c.A[i], c.k[i],
                     c.phase[i], c.theta[i]);
    std::fclose(fp);
}

}  // namespace cfdwm

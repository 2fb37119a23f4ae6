// wpf_driver -- the host program of the GB300 time step: a C++ mirror of the
// reference's `program main` (wPFAW3D.f90:2172-2325) on top of the C ABI of
// include/wpf.h.
//
//   wpf_driver <case.cfg | case.inp> [--solver fp64|mixed] [--extrapolate]
//              [--nsteps N] [--rtol R] [--quiet] [--dry-run]
//
// It reads the case as loadConfig (:264-505) or loadInput (:110-259) do, the
// well file (:402-432) and the optional .fld initial field (loadField,
// :509-557); runs the time loop (dt law :2227-2231, one wpf_step per step);
// writes the progress file <case>.dat as showProgress / doneProgress
// (:1665-1836), the GiD binary result file <case>.res as saveResult
// (:1842-2091) -- its fields packed on the device and copied to pinned memory
// on a side stream (wpf_snapshot) while the loop goes on, a writer thread
// appending them -- and the restart field <filename_last> (saveField,
// :2096-2141) plus a pressure side file <filename_last>.p that lets a
// restart resume from the same pressure, step number, step size and lagged
// taumin, so that N steps, a restart and M more steps give the fields of N+M
// continuous steps.  --nsteps N counts the steps of this run.  --dry-run
// prints the parsed case as JSON and exits (no device needed).
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "wpf.h"

namespace {

struct Well {
    int ix, iy, iz;
    double pressure, injection, phase, concent;
};

struct Case {
    int nx = 0, ny = 0, nz = 0;
    double dtime = 0.1e-6, tfac = NAN, time_start = 0.0, time_total = 0.0, time_end = 0.0;
    int n_res_out = 1, n_dat_out = 1;
    double dtime_res = 0.0, dtime_dat = 0.0;
    double epsilon = 0.0, dxw = 0.0, dx = 0.0, lx = 0.0, ly = 0.0, lz = 0.0;
    double lambda = 0.0, porosity = 0.0, rhos = 0.0, rhoa = 0.0, viscosity = 0.0, cwtp = 0.0;
    double diffusion = 0.0, b100 = 0.0, ral = 0.0, rat = 0.0, permeab_hole = 0.0, alpha = 0.0;
    double pini = 0.0;
    int ix_ref = 1, iy_ref = 1, iz_ref = 1;
    std::string filename_well, filename_init, filename_last;
    double init_permeab = 0.0, init_phase = -1.0, init_concent = 0.0;
    long nsteps = -1;          // extension key
    std::string solver;        // extension key
    std::vector<Well> wells;
};

[[noreturn]] void die(const std::string& msg) {
    fprintf(stderr, "Error: %s\n", msg.c_str());
    exit(1);
}

// Fortran list-directed real: accepts the d exponent (1.0d-3)
double num(const std::string& t) {
    std::string s = t;
    for (size_t i = 1; i + 1 < s.size(); ++i)
        if ((s[i] == 'd' || s[i] == 'D') && (isdigit((unsigned char)s[i - 1]) || s[i - 1] == '.') &&
            (isdigit((unsigned char)s[i + 1]) || s[i + 1] == '+' || s[i + 1] == '-'))
            s[i] = 'e';
    char* end = nullptr;
    const double v = strtod(s.c_str(), &end);
    if (!end || *end) throw std::invalid_argument(t);
    return v;
}

long inum(const std::string& t) {
    char* end = nullptr;
    const long v = strtol(t.c_str(), &end, 10);
    if (!end || *end) throw std::invalid_argument(t);
    return v;
}

std::vector<std::string> split(const std::string& s) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == ' ' || c == '\t' || c == ',' || c == '\r' || c == '\n') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

std::string dir_of(const std::string& p) {
    const size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string join_rel(const std::string& base, const std::string& f) {
    if (f.empty() || f[0] == '/') return f;
    return base + "/" + f;
}

void derive(Case& c) {   // wPFAW3D.f90:391-399
    if (c.n_res_out) c.dtime_res = c.time_total / c.n_res_out;
    if (c.n_dat_out) c.dtime_dat = c.time_total / c.n_dat_out;
    c.dx = c.dxw * c.epsilon;
    c.lx = c.dx * c.nx;
    c.ly = c.dx * c.ny;
    c.lz = c.dx * c.nz;
    const double b = c.rhoa / c.rhos, kc = c.cwtp * c.b100 / (1.0 - c.porosity);
    c.alpha = 0.5 / b / kc;
}

Well make_well(long ix, long iy, long iz, long wpq, double wval, double ph, double cc, const std::string& f) {
    Well w{(int)ix, (int)iy, (int)iz, 0.0, 0.0, ph, cc};
    if (wpq == 1) w.pressure = wval;
    else if (wpq == -1) w.injection = wval;
    else die("invalid data in well file: " + f);
    return w;
}

std::vector<Well> read_wells(const std::string& path) {   // :402-432
    std::ifstream in(path);
    if (!in) die("can not open well file: " + path);
    std::string line;
    std::getline(in, line);   // title
    if (!std::getline(in, line)) die("invalid data in well file: " + path);
    std::vector<Well> wells;
    try {
        const long n = inum(split(line).at(0));
        for (long w = 0; w < n; ++w) {
            if (!std::getline(in, line)) die("invalid data in well file: " + path);
            const auto t = split(line);
            wells.push_back(make_well(inum(t.at(0)), inum(t.at(1)), inum(t.at(2)), inum(t.at(3)), num(t.at(4)),
                                      num(t.at(5)), num(t.at(6)), path));
        }
    } catch (const std::exception&) {
        die("invalid data in well file: " + path);
    }
    return wells;
}

Case load_config(const std::string& path) {   // :264-505
    std::ifstream in(path);
    if (!in) die("can not open config file: " + path);
    Case c;
    std::string raw;
    while (std::getline(in, raw)) {
        std::string buf = raw;
        if (!buf.empty() && buf[0] == '#') continue;
        const size_t h = buf.find('#');
        if (h != std::string::npos) buf = buf.substr(0, h);
        const size_t e = buf.find('=');
        if (e != std::string::npos) buf[e] = ' ';
        const auto t = split(buf);
        if (t.empty()) continue;
        const std::string& k = t[0];
        try {
            auto a = [&](size_t i) -> const std::string& { return t.at(i + 1); };
            if (k == "grid") { c.nx = inum(a(0)); c.ny = inum(a(1)); c.nz = inum(a(2)); }
            else if (k == "dt") c.dtime = num(a(0));
            else if (k == "tfac") c.tfac = num(a(0));
            else if (k == "time_total") c.time_total = num(a(0));
            else if (k == "gid_output") c.n_res_out = inum(a(0));
            else if (k == "scr_output") c.n_dat_out = inum(a(0));
            else if (k == "w") c.epsilon = num(a(0));
            else if (k == "dxw") c.dxw = num(a(0));
            else if (k == "lambda") c.lambda = num(a(0));
            else if (k == "poro") c.porosity = num(a(0));
            else if (k == "rhos") c.rhos = num(a(0));
            else if (k == "rhoa") c.rhoa = num(a(0));
            else if (k == "visco") c.viscosity = num(a(0));
            else if (k == "cwtp") c.cwtp = num(a(0));
            else if (k == "D") c.diffusion = num(a(0));
            else if (k == "b100") c.b100 = num(a(0));
            else if (k == "ral") c.ral = num(a(0));
            else if (k == "rat") c.rat = num(a(0));
            else if (k == "kwh") c.permeab_hole = num(a(0));
            else if (k == "pini") c.pini = num(a(0));
            else if (k == "ref") { c.ix_ref = inum(a(0)); c.iy_ref = inum(a(1)); c.iz_ref = inum(a(2)); }
            else if (k == "well") c.filename_well = a(0);
            else if (k == "init") {
                try {
                    const double p = num(a(0)), q = num(a(1)), r = num(a(2));
                    c.init_permeab = p; c.init_phase = q; c.init_concent = r;
                } catch (const std::exception&) {
                    c.filename_init = a(0);
                }
            }
            else if (k == "last") c.filename_last = a(0);
            else if (k == "nsteps") c.nsteps = inum(a(0));
            else if (k == "solver") c.solver = a(0);
            else die("unknown key in config file: " + path + ": " + k);
        } catch (const std::exception&) {
            die("broken line in config file: " + path + ": " + raw);
        }
    }
    derive(c);
    if (!(c.tfac == c.tfac)) die("tfac is required (the reference leaves it uninitialised)");
    const std::string base = dir_of(path);
    c.wells = read_wells(join_rel(base, c.filename_well));
    if (!c.filename_init.empty()) c.filename_init = join_rel(base, c.filename_init);
    return c;
}

// loadInput (:110-259): a fixed sequence of comment records and list-directed reads
Case load_input(const std::string& path) {
    std::ifstream in(path);
    if (!in) die("can not open input file: " + path);
    std::vector<std::string> lines;
    std::string l;
    while (std::getline(in, l)) lines.push_back(l);
    size_t pos = 0;
    auto skip = [&](int n) { pos += n; };
    std::vector<std::string> pend;
    auto read = [&](size_t n) {   // list-directed: continue on the next records if needed
        std::vector<std::string> out;
        while (out.size() < n) {
            if (pos >= lines.size()) die("invalid data in input file: " + path);
            for (auto& t : split(lines[pos])) out.push_back(t);
            ++pos;
        }
        out.resize(n);
        return out;
    };
    Case c;
    try {
        skip(5);
        auto v = read(3); c.nx = inum(v[0]); c.ny = inum(v[1]); c.nz = inum(v[2]);
        skip(1); v = read(2); c.dtime = num(v[0]); c.tfac = num(v[1]);
        skip(1); v = read(4); c.time_start = num(v[0]); c.time_end = num(v[1]);
        c.n_res_out = inum(v[2]); c.n_dat_out = inum(v[3]);
        skip(2); v = read(2); c.epsilon = num(v[0]); c.dxw = num(v[1]);
        skip(1); c.lambda = num(read(1)[0]);
        skip(2); c.porosity = num(read(1)[0]);
        skip(1); v = read(2); c.rhos = num(v[0]); c.rhoa = num(v[1]);
        skip(1); c.viscosity = num(read(1)[0]);
        skip(1); c.cwtp = num(read(1)[0]);
        skip(1); c.diffusion = num(read(1)[0]);
        skip(2); c.b100 = num(read(1)[0]);
        skip(1); v = read(2); c.ral = num(v[0]); c.rat = num(v[1]);
        skip(1); c.permeab_hole = num(read(1)[0]);
        skip(1); c.pini = num(read(1)[0]);
        skip(1); v = read(3); c.ix_ref = inum(v[0]); c.iy_ref = inum(v[1]); c.iz_ref = inum(v[2]);
        skip(2);
        const long nw = inum(read(1)[0]);
        for (long w = 0; w < nw; ++w) {
            v = read(7);
            c.wells.push_back(make_well(inum(v[0]), inum(v[1]), inum(v[2]), inum(v[3]), num(v[4]), num(v[5]),
                                        num(v[6]), path));
        }
        skip(2); c.init_permeab = num(read(1)[0]);
        skip(1); c.init_phase = num(read(1)[0]);
        skip(1); c.init_concent = num(read(1)[0]);
    } catch (const std::exception&) {
        die("invalid data in input file: " + path);
    }
    c.time_total = c.time_end - c.time_start;
    derive(c);
    return c;
}

// ---- .fld restart file (:509-557, :2096-2141) ------------------------------------
// The pressure side file <last>.p: the G halo values of the pressure, then this
// trailer (no counterpart in the reference, which restarts at itime 0 with the
// configured dt): the last step number, its dt and the lagged taumin.
static const char kTrailerTag[8] = {'W', 'P', 'F', 'S', 'T', 'E', 'P', '1'};
struct StepTrailer {
    char tag[8];
    double itime, dtime, taumin;
};

struct FldHead {
    char magic[8];
    char version[8];
    double time;
    int16_t nx, ny, nz, pad;
};
static_assert(sizeof(FldHead) == 32, "fld header is 32 bytes");

void read_fld(const Case& c, double* time, std::vector<double>& kr, std::vector<double>& ph,
              std::vector<double>& cc) {
    FILE* f = fopen(c.filename_init.c_str(), "rb");
    if (!f) die("can not open field file: " + c.filename_init);
    FldHead h;
    if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "wPFAWHFG", 8))
        die("invalid magic in field file: " + c.filename_init);
    if (h.nx != c.nx || h.ny != c.ny || h.nz != c.nz) die("invalid grid in field file: " + c.filename_init);
    *time = h.time;
    const size_t n = (size_t)c.nx * c.ny * c.nz;
    kr.resize(n); ph.resize(n); cc.resize(n);
    if (fread(kr.data(), 8, n, f) != n || fread(ph.data(), 8, n, f) != n || fread(cc.data(), 8, n, f) != n)
        die("short field file: " + c.filename_init);
    fclose(f);
}

void write_fld(const std::string& path, const Case& c, double time, const double* kr, const double* ph,
               const double* cc) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) die("can not create field file: " + path);
    FldHead h;
    memcpy(h.magic, "wPFAWHFG", 8);
    memcpy(h.version, "20250304", 8);
    h.time = time;
    h.nx = (int16_t)c.nx; h.ny = (int16_t)c.ny; h.nz = (int16_t)c.nz; h.pad = 0;
    const size_t n = (size_t)c.nx * c.ny * c.nz;
    fwrite(&h, sizeof h, 1, f);
    fwrite(kr, 8, n, f);
    fwrite(ph, 8, n, f);
    fwrite(cc, 8, n, f);
    fclose(f);
}

// ---- Fortran edit descriptors --------------------------------------------------------
std::string es(double v, int w, int d) {   // ESw.d (a three-digit exponent drops the E)
    char buf[64];
    snprintf(buf, sizeof buf, "%.*E", d, v);
    std::string s(buf);
    const size_t k = s.find('E');
    const int e = atoi(s.c_str() + k + 1);
    char eb[16];
    if (abs(e) < 100) snprintf(eb, sizeof eb, "E%c%02d", e < 0 ? '-' : '+', abs(e));
    else snprintf(eb, sizeof eb, "%c%03d", e < 0 ? '-' : '+', abs(e));
    s = s.substr(0, k) + eb;
    if ((int)s.size() > w) return std::string(w, '*');
    return std::string(w - s.size(), ' ') + s;
}
std::string fx(double v, int w, int d) {
    char buf[64];
    snprintf(buf, sizeof buf, "%*.*f", w, d, v);
    std::string s(buf);
    return (int)s.size() > w ? std::string(w, '*') : s;
}
std::string ix(long v, int w) {
    char buf[32];
    snprintf(buf, sizeof buf, "%*ld", w, v);
    std::string s(buf);
    return (int)s.size() > w ? std::string(w, '*') : s;
}

// ---- showProgress (.dat) -----------------------------------------------------------------
struct Progress {
    FILE* f = nullptr;
    double pv = 0.0;
    std::chrono::steady_clock::time_point t0;
    std::clock_t c0 = 0;
    bool echo = true;

    void first(const Case& c, const wpf_diag& d, const std::string& path) {
        f = fopen(path.c_str(), "w");
        if (!f) die("can not create progress file: " + path);
        t0 = std::chrono::steady_clock::now();
        c0 = std::clock();
        pv = d.pv;
        const double xchl = c.cwtp * c.b100 * c.rhoa / c.rhos, b = c.rhoa / c.rhos;
        const double kc = c.cwtp * c.b100 / (1.0 - c.porosity);
        auto w = [&](const std::string& s) { fprintf(f, "%s\n", s.c_str()); };
        w(" ***** CALCULATION SUMMARY FOR PFACID PROGRAM *****");
        w(" /// Input data ///");
        w(" *** Grid data");
        w("   Num of grids, nx,ny,nz =" + ix(c.nx, 6) + ix(c.ny, 6) + ix(c.nz, 6));
        w("   Grid size, dx       =" + es(c.dx, 14, 6) + " [m]");
        w("   Core length, Lx, Ly, Lz =" + fx(c.lx, 10, 4) + fx(c.ly, 10, 4) + fx(c.lz, 10, 4) + " [m]");
        w(" *** Rock and fluid data");
        w("   acid con., cwtp      =" + fx(c.cwtp, 12, 4) + " [kg HCl/kg solution]");
        w("   acid density, rhoa   =" + fx(c.rhoa, 12, 1) + " [kg/m3]");
        w("   rock density, rhos   =" + fx(c.rhos, 12, 1) + " [kg/m3]");
        w("   viscosity, visco     =" + es(c.viscosity, 14, 6) + " [Pa*s]");
        w("   rock porosity, poro  =" + fx(c.porosity, 12, 6) + " [dec]");
        w("   diffusivity coef. ,d =" + es(c.diffusion, 12, 4) + " [m2/s]");
        w("   gravimetric dissolving power, b100 =" + fx(c.b100, 8, 3) + " [kg CaCO3/kg HCl]");
        w("   volumetric dissolving power, Xacid =" + fx(xchl, 8, 3) + " [m3 CaCO3/m3 HCl]");
        w(" *** Phase-field related parameters");
        w("   lambda =" + fx(c.lambda, 12, 6) + " [-]");
        w("   kc     =" + fx(kc, 12, 6) + " [-]");
        w("   b      =" + fx(b, 12, 6) + " [-]");
        w("   alpha  =" + fx(c.alpha, 12, 6) + " [-]");
        w(" *** Injection data");
        w("   time step size, dt     =" + es(c.dtime, 12, 4) + " [s]");
        w("   initial pressure, pini =" + es(c.pini, 12, 4) + " [m/s]");
        w(" pore volume =" + es(pv, 20, 6) + " [m3]");
        w("");
        w("");
        w("/// SIMULATION RESULTS ///");
        w(std::string(13, ' ') + "ITIME" + std::string(2, ' ') + "TIME" + std::string(15, ' ') + "PVINJ" +
          std::string(13, ' ') + "WELL_PRESS" + std::string(10, ' ') + "WH_LENGTH" + std::string(10, ' ') +
          "INJ_ACID" + std::string(11, ' ') + "DISSOLVED_CaCO3" + std::string(10, ' ') + "DISS.CaCO3_c");
        w(std::string(13, ' ') + "(-)" + std::string(4, ' ') + "(sec)" + std::string(15, ' ') + "(v/v)" +
          std::string(15, ' ') + "(Pa)" + std::string(16, ' ') + "(m)" + std::string(14, ' ') + "(m3/m)" +
          std::string(14, ' ') + "(m3/m)" + std::string(14, ' ') + "(m3/m)");
        std::string dash = std::string(5, ' ') + "-----" + std::string(2, ' ');
        for (int q = 0; q < 6; ++q) dash += "   --------------   ";
        w(dash);
        if (echo) {
            printf("*** 3D Phase-Field Acid Wormholing Model, wPFAW3D ***\n\n");
            printf(" # of equations,     neq =%12ld\n", (long)c.nx * c.ny * c.nz);
            printf(" pore volume =%s [m3]\n", es(pv, 20, 6).c_str());
            printf("   ITIME     TIME        PVINJ     MAX_PHI MIN_PHI  MAX_C   MIN_C     PINJ         RWH         DT\n");
        }
    }

    void write(const Case& c, const wpf_diag& d, double time, long itime, double pinj, double dt,
               const std::string& path) {
        if (!f) first(c, d, path);
        const double xchl = c.cwtp * c.b100 * c.rhoa / c.rhos;
        double qinj = 0.0;
        for (const Well& w : c.wells)
            if (w.injection != 0.0) qinj += w.injection;
        const double vacid = qinj * time, vcaco3 = qinj * time * xchl;
        std::string row = " " + ix(itime, 8) + " ";
        for (double v : {time, vacid / pv, pinj, d.rwhmax, vacid, vcaco3, d.vcal}) row += es(v, 20, 10);
        fprintf(f, "%s\n", row.c_str());
        fflush(f);
        if (echo)
            printf("%s%s%s %s%s%s%s%s%s%s\n", ix(itime, 8).c_str(), es(time, 13, 5).c_str(),
                   es(vacid / pv, 11, 3).c_str(), fx(d.phase_max, 8, 3).c_str(), fx(d.phase_min, 8, 3).c_str(),
                   fx(d.concent_max, 8, 3).c_str(), fx(d.concent_min, 8, 3).c_str(), es(pinj, 13, 5).c_str(),
                   es(d.rwhmax, 12, 4).c_str(), es(dt, 10, 2).c_str());
    }

    void done() {   // doneProgress
        if (!f) return;
        const double cpu = (double)(std::clock() - c0) / CLOCKS_PER_SEC / 60.0;
        const double wall =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / 60.0;
        fprintf(f, "\nCPU time =%s [min]\nCal time =%s [min]\n", es(cpu, 12, 4).c_str(), es(wall, 12, 4).c_str());
        fclose(f);
        f = nullptr;
    }
};

// ---- saveResult (GiD binary .res) ------------------------------------------------------------
struct GidResult {
    FILE* f = nullptr;
    long n = 0;
    float* snap = nullptr;     // pinned, 4 * n floats (wpf_snapshot)
    std::thread writer;
    wpf_handle* h = nullptr;

    void str(const std::string& s) {
        const int32_t len = (int32_t)s.size() + 1;
        fwrite(&len, 4, 1, f);
        fwrite(s.c_str(), 1, s.size() + 1, f);
    }

    void open(const std::string& path, const Case& c, wpf_handle* hh) {
        h = hh;
        f = fopen(path.c_str(), "wb");
        if (!f) die("can not create result file: " + path);
        n = (long)c.nx * c.ny * c.nz;
        if (wpf_host_alloc(4 * 4 * n, (void**)&snap)) die("wpf_host_alloc failed");
        const int32_t bom = 0x091d;
        fwrite(&bom, 4, 1, f);
        str("GiDPostEx1.1");
        str("MESH \"quadmesh\" dimension 3 ElemType Hexahedra Nnode 8");
        str("# color 0.7 0.7 0.4");
        str("Unit \"m\"");
        str("Coordinates -1 Indexed");
        const long NX = c.nx + 1, NY = c.ny + 1;
        auto m = [&](long a, long b, long q) { return (int32_t)(a + b * NX + q * NX * NY + 1); };
        struct __attribute__((packed)) Node { int32_t i; float x, y, z; };
        std::vector<Node> row((size_t)NX);
        for (long z = 0; z <= c.nz; ++z)
            for (long y = 0; y <= c.ny; ++y) {
                for (long x = 0; x <= c.nx; ++x)
                    row[(size_t)x] = Node{m(x, y, z), (float)(x * c.dx), (float)(y * c.dx), (float)(z * c.dx)};
                fwrite(row.data(), sizeof(Node), row.size(), f);
            }
        str("End Coordinates");
        str("Elements -1 Indexed");
        struct __attribute__((packed)) Elem { int32_t i, nid[8], conn; };
        std::vector<Elem> er((size_t)c.nx);
        for (long z = 0; z < c.nz; ++z)
            for (long y = 0; y < c.ny; ++y) {
                for (long x = 0; x < c.nx; ++x) {
                    Elem& e = er[(size_t)x];
                    e.i = (int32_t)(x + y * c.nx + z * (long)c.nx * c.ny + 1);
                    e.nid[0] = m(x, y, z);         e.nid[1] = m(x + 1, y, z);
                    e.nid[2] = m(x + 1, y + 1, z); e.nid[3] = m(x, y + 1, z);
                    e.nid[4] = m(x, y, z + 1);     e.nid[5] = m(x + 1, y, z + 1);
                    e.nid[6] = m(x + 1, y + 1, z + 1); e.nid[7] = m(x, y + 1, z + 1);
                    e.conn = 1;
                }
                fwrite(er.data(), sizeof(Elem), er.size(), f);
            }
        str("End Elements");
        str("GaussPoints \"Cell_Center\" ElemType Hexahedra");
        str("Number Of Gauss Points: 1");
        str("Natural Coordinates: Given");
        const float zeros[3] = {0.f, 0.f, 0.f};
        fwrite(zeros, 4, 3, f);
        str("End GaussPoints");
        fflush(f);
    }

    void blocks(double time) {   // runs on the writer thread once the snapshot has landed
        if (wpf_snapshot_wait(h)) die("wpf_snapshot_wait failed");
        static const char* names[4] = {"Pressure", "Phase-field", "Concentration", "Permeability"};
        static const char* units[4] = {"Pa", "-", "-", "-"};
        struct __attribute__((packed)) Val { int32_t i; float v; };
        std::vector<Val> vals((size_t)n);
        for (int q = 0; q < 4; ++q) {
            str("Result \"" + std::string(names[q]) + "\" \"Analysis\" " + es(time, 12, 5) +
                " Scalar OnGaussPoints \"Cell_Center\"");
            str(std::string("Unit \"") + units[q] + "\"");
            str("Values -1 Indexed");
            for (long e = 0; e < n; ++e) vals[(size_t)e] = Val{(int32_t)(e + 1), snap[q * n + e]};
            fwrite(vals.data(), sizeof(Val), vals.size(), f);
            const int32_t end = -1;
            fwrite(&end, 4, 1, f);
            str("End Values");
        }
        fflush(f);
    }

    void save(double time) {
        if (writer.joinable()) writer.join();
        if (wpf_snapshot(h, snap)) die("wpf_snapshot failed");
        writer = std::thread([this, time]() { blocks(time); });
    }

    void done() {   // doneResult
        if (writer.joinable()) writer.join();
        if (f) fclose(f);
        f = nullptr;
        if (snap) wpf_host_free(snap);
        snap = nullptr;
    }
};

void print_case_json(const Case& c) {
    printf("{\"nx\": %d, \"ny\": %d, \"nz\": %d, \"dtime\": %.17g, \"tfac\": %.17g, \"time_start\": %.17g, "
           "\"time_total\": %.17g, \"time_end\": %.17g, \"n_res_out\": %d, \"n_dat_out\": %d, "
           "\"dtime_res\": %.17g, \"dtime_dat\": %.17g, \"epsilon\": %.17g, \"dx\": %.17g, "
           "\"lambda_\": %.17g, \"porosity\": %.17g, \"rhos\": %.17g, \"rhoa\": %.17g, \"viscosity\": %.17g, "
           "\"cwtp\": %.17g, \"diffusion\": %.17g, \"b100\": %.17g, \"ral\": %.17g, \"rat\": %.17g, "
           "\"permeab_hole\": %.17g, \"alpha\": %.17g, \"pini\": %.17g, \"ix_ref\": %d, \"iy_ref\": %d, "
           "\"iz_ref\": %d, \"init_permeab\": %.17g, \"init_phase\": %.17g, \"init_concent\": %.17g, "
           "\"filename_init\": \"%s\", \"nsteps\": %ld, \"wells\": [",
           c.nx, c.ny, c.nz, c.dtime, c.tfac, c.time_start, c.time_total, c.time_end, c.n_res_out, c.n_dat_out,
           c.dtime_res, c.dtime_dat, c.epsilon, c.dx, c.lambda, c.porosity, c.rhos, c.rhoa, c.viscosity, c.cwtp,
           c.diffusion, c.b100, c.ral, c.rat, c.permeab_hole, c.alpha, c.pini, c.ix_ref, c.iy_ref, c.iz_ref,
           c.init_permeab, c.init_phase, c.init_concent, c.filename_init.c_str(), c.nsteps);
    for (size_t w = 0; w < c.wells.size(); ++w) {
        const Well& x = c.wells[w];
        printf("%s[%d, %d, %d, %.17g, %.17g, %.17g, %.17g]", w ? ", " : "", x.ix, x.iy, x.iz, x.pressure,
               x.injection, x.phase, x.concent);
    }
    printf("]}\n");
}

void check(int rc, const char* what) {
    if (rc) die(std::string(what) + ": " + wpf_strerror(rc));
}

}  // namespace

int main(int argc, char** argv) {
    std::string file, solver;
    bool extrapolate = false, quiet = false, dry = false;
    long nsteps = -1;
    double rtol = 1e-8;
    for (int a = 1; a < argc; ++a) {
        const std::string s = argv[a];
        if (s == "--solver" && a + 1 < argc) solver = argv[++a];
        else if (s == "--extrapolate") extrapolate = true;
        else if (s == "--nsteps" && a + 1 < argc) nsteps = atol(argv[++a]);
        else if (s == "--rtol" && a + 1 < argc) rtol = atof(argv[++a]);
        else if (s == "--quiet") quiet = true;
        else if (s == "--dry-run") dry = true;
        else if (file.empty()) file = s;
        else die("unexpected argument: " + s);
    }
    if (file.empty()) die("no input file is given.");
    Case c;
    size_t i = file.find(".inp");
    if (i != std::string::npos) {
        c = load_input(file);
        c.filename_last = file.substr(0, i) + ".last.fld";
    } else {
        i = file.find(".cfg");
        if (i == std::string::npos) die("input file is neither inp or cfg.");
        c = load_config(file);
    }
    std::vector<double> kr0, ph0, cc0;
    if (!c.filename_init.empty()) read_fld(c, &c.time_start, kr0, ph0, cc0);
    c.time_end = c.time_start + c.time_total;
    if (nsteps < 0) nsteps = c.nsteps;
    if (solver.empty()) solver = c.solver.empty() ? "fp64" : c.solver;
    if (dry) {
        print_case_json(c);
        return 0;
    }
    const std::string stem = file.substr(0, i);
    const std::string fdat = stem + ".dat", fres = stem + ".res";

    // initial fields as loadConfig / loadInput build them (:464-496)
    const long NX = c.nx + 2, NY = c.ny + 2, NZ = c.nz + 2, G = NX * NY * NZ;
    std::vector<double> kr((size_t)G, c.init_permeab), ph((size_t)G, c.init_phase), cc((size_t)G, c.init_concent),
        pr((size_t)G, c.pini);
    auto at = [&](long x, long y, long z) { return (size_t)(x + NX * (y + NY * z)); };
    for (const Well& w : c.wells)
        if (1 <= w.ix && w.ix <= c.nx && 1 <= w.iy && w.iy <= c.ny && 1 <= w.iz && w.iz <= c.nz) {
            ph[at(w.ix, w.iy, w.iz)] = w.phase;
            cc[at(w.ix, w.iy, w.iz)] = w.concent;
        }
    if (!kr0.empty())
        for (long z = 1; z <= c.nz; ++z)
            for (long y = 1; y <= c.ny; ++y)
                for (long x = 1; x <= c.nx; ++x) {
                    const size_t d = (size_t)((x - 1) + c.nx * ((y - 1) + (long)c.ny * (z - 1)));
                    kr[at(x, y, z)] = kr0[d];
                    ph[at(x, y, z)] = ph0[d];
                    cc[at(x, y, z)] = cc0[d];
                }
    // a pressure side file written with the restart field resumes the pressure
    // too, and, when it carries the step trailer, the step count, the step size
    // and the lagged taumin of the dt law (the reference restarts at itime 0)
    long itime_resume = 0;
    double dt_resume = 0.0, taumin_resume = 0.0;
    if (!c.filename_init.empty()) {
        FILE* pf = fopen((c.filename_init + ".p").c_str(), "rb");
        if (pf) {
            std::vector<double> p0((size_t)G);
            if (fread(p0.data(), 8, (size_t)G, pf) == (size_t)G) {
                pr = p0;
                StepTrailer t;
                if (fread(&t, sizeof t, 1, pf) == 1 && !memcmp(t.tag, kTrailerTag, 8)) {
                    itime_resume = (long)t.itime;
                    dt_resume = t.dtime;
                    taumin_resume = t.taumin;
                }
            }
            fclose(pf);
        }
    }

    wpf_params prm;
    memset(&prm, 0, sizeof prm);
    prm.nx = c.nx; prm.ny = c.ny; prm.nz = c.nz;
    prm.ix_ref = c.ix_ref; prm.iy_ref = c.iy_ref; prm.iz_ref = c.iz_ref;
    prm.dx = c.dx; prm.epsilon = c.epsilon; prm.lambda = c.lambda; prm.porosity = c.porosity;
    prm.viscosity = c.viscosity; prm.diffusion = c.diffusion; prm.ral = c.ral; prm.rat = c.rat;
    prm.permeab_hole = c.permeab_hole; prm.alpha = c.alpha; prm.tfac = c.tfac;
    wpf_handle* h = nullptr;
    check(wpf_create(&prm, &h), "wpf_create");
    std::vector<wpf_well> ws;
    for (const Well& w : c.wells) ws.push_back(wpf_well{w.ix, w.iy, w.iz, 0, w.pressure, w.injection, w.phase, w.concent});
    check(wpf_set_wells(h, ws.data(), (int32_t)ws.size()), "wpf_set_wells");
    check(wpf_upload(h, kr.data(), ph.data(), cc.data(), pr.data()), "wpf_upload");
    wpf_solver_opts o;
    check(wpf_get_solver(h, &o), "wpf_get_solver");
    o.mode = solver == "mixed" ? WPF_SOLVER_MIXED : WPF_SOLVER_FP64;
    o.rtol = rtol;
    if (extrapolate) o.flags |= WPF_SOLVER_EXTRAPOLATE;
    check(wpf_set_solver(h, &o), "wpf_set_solver");

    long itime = itime_resume;
    double time = c.time_start;
    double time_res = time + c.dtime_res, time_dat = time + c.dtime_dat;
    double dt = itime_resume > 0 ? dt_resume : c.dtime;
    if (itime_resume > 0 && taumin_resume > 0.0) check(wpf_set_taumin(h, taumin_resume), "wpf_set_taumin");
    const long itime0 = itime;
    Progress prog;
    prog.echo = !quiet;
    GidResult res;
    res.open(fres, c, h);
    auto p_at = [&](int x, int y, int z) {   // getPressure
        if (!(1 <= x && x <= c.nx && 1 <= y && y <= c.ny && 1 <= z && z <= c.nz)) return 0.0;
        std::vector<double> tmp((size_t)G);
        check(wpf_download(h, nullptr, nullptr, tmp.data(), nullptr, nullptr, nullptr, nullptr), "wpf_download");
        return tmp[at(x, y, z)];
    };
    wpf_diag d;
    res.save(time);
    check(wpf_reduce(h, &d), "wpf_reduce");
    prog.write(c, d, time, itime, p_at(1, 1, 1), dt, fdat);
    wpf_step_stats st;
    while (time < c.time_end && (nsteps < 0 || itime - itime0 < nsteps)) {
        ++itime;
        const int rc = wpf_step(h, (int32_t)itime, &dt, &st);
        if (rc && rc != WPF_ERR_NOT_CONVERGED) check(rc, "wpf_step");
        time += dt;
        if (time > time_dat) {
            check(wpf_reduce(h, &d), "wpf_reduce");
            prog.write(c, d, time, itime, d.pressure_ref, dt, fdat);
            time_dat += c.dtime_dat;
        }
        if (time > time_res) {
            res.save(time);
            time_res += c.dtime_res;
        }
    }
    prog.done();
    res.done();
    if (!c.filename_last.empty()) {   // saveField (+ the pressure side file)
        std::vector<double> P((size_t)G), Q((size_t)G), R((size_t)G);
        check(wpf_download(h, P.data(), Q.data(), R.data(), nullptr, nullptr, nullptr, nullptr), "wpf_download");
        const size_t n = (size_t)c.nx * c.ny * c.nz;
        std::vector<double> a(n), b(n), e(n);
        for (long z = 1; z <= c.nz; ++z)
            for (long y = 1; y <= c.ny; ++y)
                for (long x = 1; x <= c.nx; ++x) {
                    const size_t q = (size_t)((x - 1) + c.nx * ((y - 1) + (long)c.ny * (z - 1)));
                    a[q] = kr[at(x, y, z)];
                    b[q] = P[at(x, y, z)];
                    e[q] = Q[at(x, y, z)];
                }
        write_fld(c.filename_last, c, time, a.data(), b.data(), e.data());
        FILE* pf = fopen((c.filename_last + ".p").c_str(), "wb");
        if (pf) {
            StepTrailer t;
            memcpy(t.tag, kTrailerTag, 8);
            t.itime = (double)itime;
            t.dtime = dt;
            check(wpf_get_taumin(h, &t.taumin), "wpf_get_taumin");
            fwrite(R.data(), 8, (size_t)G, pf);
            fwrite(&t, sizeof t, 1, pf);
            fclose(pf);
        }
    }
    check(wpf_destroy(h), "wpf_destroy");
    if (!quiet) printf("\n%ld steps, time %s\n", itime, es(time, 12, 5).c_str());
    return 0;
}

// state_io.cpp -- configuration and checkpoint files of PIMD-F90 (host code, no device work).
//
// Restates the file formats of InputOutput.f90:
//   * the configuration header of read_and_initialize_all_nodes (InputOutput.f90:67-116):
//     ".img" images start with '(2i10)' Natoms, Nbeads and '(f12.6,2x,f12.6,3(1x,f12.6))' time
//     and box; ".xyz" files hold the box and the atom count in one of three layouts (box line
//     then count, count then box line, or count and box on one line);
//   * read_coords_and_init (InputOutput.f90:422-446): list-directed "symbol x y z" records,
//     read_method 0 (all O, then the H pairs) or 1 (O H H ...), the coordinates shifted by the
//     mean that the read_method 1 loop accumulates (read_method 0 accumulates none);
//   * save_XYZ (InputOutput.f90:948-981): '(i10)' Natoms, a blank record, '(a2,3(1x,f12.6))';
//   * save_checkpoint / load_checkpoint (InputOutput.f90:987-1074): per molecule and atom all
//     beads as '(a2,6(1x,f12.6))' position and velocity (momentum / mass), then the bead and
//     global Nose-Hoover chain velocities as list-directed records; the loader multiplies the
//     velocities by the masses, forms the centroid and applies the centroid-following PBC shift
//     (main_stuff.f90:107-125).
// Fixed-width fields are written and read as a Fortran F edit descriptor does: rounded to the
// stated decimals, asterisks when the number does not fit, blanks in an input field ignored and
// a field without a decimal point scaled by 10^-d. List-directed reals are written as
// gfortran writes REAL(8) (one blank, then G25.17E3) and read in free form.
//
// Deviation: the reference tries the box-line-first layout before the others, so a file whose
// first record holds the count and the box (input_coords/input_512.xyz) reads the count as a box
// edge there and fails on the next record; this reader picks the layout by the number of values
// on the first record (3: box first, 1: count first, 4: count and box).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimd_gb300.h"

namespace {

struct LineReader {
    FILE *f = nullptr;
    std::string line;
    explicit LineReader(const char *path) { f = std::fopen(path, "r"); }
    ~LineReader() {
        if (f) std::fclose(f);
    }
    bool next() {  // one record without its line end
        line.clear();
        int c;
        bool any = false;
        while ((c = std::fgetc(f)) != EOF) {
            any = true;
            if (c == '\n') break;
            line.push_back((char)c);
        }
        if (!line.empty() && line.back() == '\r') line.pop_back();
        return any;
    }
};

// list-directed items of one record: blanks, commas and tabs separate
std::vector<std::string> split_items(const std::string &s) {
    std::vector<std::string> out;
    std::string cur;
    for (char ch : s) {
        if (ch == ' ' || ch == ',' || ch == '\t') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

// a Fortran real in free form (D exponents accepted)
bool parse_real(std::string s, double *v) {
    for (char &c : s)
        if (c == 'd' || c == 'D') c = 'E';
    char *end = nullptr;
    *v = std::strtod(s.c_str(), &end);
    return end && *end == '\0' && !s.empty();
}
bool parse_int(const std::string &s, int *v) {
    char *end = nullptr;
    const long x = std::strtol(s.c_str(), &end, 10);
    if (!end || *end != '\0' || s.empty()) return false;
    *v = (int)x;
    return true;
}

// next record with at least one list-directed item (list-directed input continues over blank
// records)
bool next_items(LineReader &r, std::vector<std::string> &items) {
    while (r.next()) {
        items = split_items(r.line);
        if (!items.empty()) return true;
    }
    return false;
}

// Fw.d input edit of columns [pos, pos + w) of a record
bool read_f(const std::string &rec, size_t pos, int w, int d, double *v) {
    std::string s;
    for (size_t i = pos; i < pos + (size_t)w && i < rec.size(); i++)
        if (rec[i] != ' ') s.push_back(rec[i]);
    if (s.empty()) {
        *v = 0.0;
        return true;
    }
    const bool point = s.find('.') != std::string::npos;
    if (!parse_real(s, v)) return false;
    if (!point) {
        // no decimal point: the digits carry d implied decimals; an exponent still applies
        const size_t e = s.find_first_of("eEdD");
        double mant;
        if (!parse_real(s.substr(0, e), &mant)) return false;
        const double expo = (e == std::string::npos) ? 0.0 : std::strtod(s.substr(e + 1).c_str(), nullptr);
        *v = mant * std::pow(10.0, expo - d);
    }
    return true;
}

// Fw.d output edit
std::string write_f(double v, int w, int d) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%*.*f", w, d, v);
    std::string s(buf);
    if ((int)s.size() > w) return std::string((size_t)w, '*');
    return s;
}
std::string write_i(long v, int w) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%*ld", w, v);
    std::string s(buf);
    if ((int)s.size() > w) return std::string((size_t)w, '*');
    return s;
}

// one list-directed REAL(8) item as gfortran writes it: a blank, then G25.17E3
std::string write_ld(double v) {
    const int w = 25, d = 17, e = 3;
    const double a = std::fabs(v);
    char buf[96];
    std::string s;
    // F form when 0.1 <= |v| < 10^d after rounding to d significant digits (and for zero)
    bool fform = false;
    int k = 0;
    if (a == 0.0) {
        fform = true;
        k = 1;
    } else if (std::isfinite(a)) {
        std::snprintf(buf, sizeof buf, "%.*e", d - 1, a);  // rounded to d significant digits
        const int ex = std::atoi(std::strchr(buf, 'e') + 1);
        if (ex >= -1 && ex < d) {
            fform = true;
            k = ex + 1;  // digits before the decimal point
        }
    }
    if (fform) {
        std::snprintf(buf, sizeof buf, "%*.*f", w - (e + 2), d - k, v);
        s = buf;
        s += std::string((size_t)(e + 2), ' ');
    } else if (std::isfinite(a)) {
        std::snprintf(buf, sizeof buf, "%.*E", d - 1, v);
        std::string m(buf);
        const size_t p = m.find('E');
        const int ex = std::atoi(m.c_str() + p + 1);
        char eb[16];
        std::snprintf(eb, sizeof eb, "E%c%0*d", ex < 0 ? '-' : '+', e, std::abs(ex));
        m = m.substr(0, p) + eb;
        std::snprintf(buf, sizeof buf, "%*s", w, m.c_str());
        s = buf;
    } else {
        std::snprintf(buf, sizeof buf, "%*s", w, std::isnan(v) ? "NaN" : (v < 0 ? "-Infinity" : "Infinity"));
        s = buf;
    }
    return " " + s;
}

bool ends_with(const char *s, const char *suf) {
    const size_t n = std::strlen(s), m = std::strlen(suf);
    return n >= m && std::strcmp(s + n - m, suf) == 0;
}

double anint(double x) { return std::round(x); }  // round half away from zero, as Fortran ANINT

// '(a2,6(1x,f12.6))' record: symbol, 3 positions, 3 velocities
bool read_image_atom(const std::string &rec, double *x, double *v) {
    for (int c = 0; c < 6; c++) {
        double val;
        if (!read_f(rec, 2 + (size_t)c * 13 + 1, 12, 6, &val)) return false;
        (c < 3 ? x[c] : v[c - 3]) = val;
    }
    return true;
}

}  // namespace

extern "C" {

int pimd_read_config_header(const char *path, int *natoms, int *nbeads, double *time, double *box) {
    if (!path || !natoms || !box) return PIMD_ERR_ARG;
    LineReader r(path);
    if (!r.f) return PIMD_ERR_ARG;
    if (nbeads) *nbeads = 0;
    if (time) *time = 0.0;
    if (ends_with(path, ".img")) {
        // '(2i10)' Natoms, Nbeads, then '(f12.6,2x,f12.6,3(1x,f12.6))' time, box
        if (!r.next()) return PIMD_ERR_ARG;
        const std::string h = r.line;
        std::vector<std::string> it = split_items(h.substr(0, std::min<size_t>(h.size(), 20)));
        int nb = 0;
        if (it.size() != 2 || !parse_int(it[0], natoms) || !parse_int(it[1], &nb)) return PIMD_ERR_ARG;
        if (nbeads) *nbeads = nb;
        if (!r.next()) return PIMD_ERR_ARG;
        double tt;
        if (!read_f(r.line, 0, 12, 6, &tt)) return PIMD_ERR_ARG;
        for (int c = 0; c < 3; c++)  // box(1) after 2x, the others after 1x each
            if (!read_f(r.line, 14 + (size_t)c * 13, 12, 6, &box[c])) return PIMD_ERR_ARG;
        if (time) *time = tt;
        return *natoms > 0 && *natoms % 3 == 0 ? PIMD_OK : PIMD_ERR_ARG;
    }
    if (!ends_with(path, ".xyz")) return PIMD_ERR_ARG;
    std::vector<std::string> a, b;
    if (!next_items(r, a)) return PIMD_ERR_ARG;
    bool ok = false;
    if (a.size() >= 4) {  // Natoms and box on one record
        ok = parse_int(a[0], natoms) && parse_real(a[1], &box[0]) && parse_real(a[2], &box[1]) &&
             parse_real(a[3], &box[2]);
    } else if (a.size() == 3) {  // box record, then Natoms
        ok = parse_real(a[0], &box[0]) && parse_real(a[1], &box[1]) && parse_real(a[2], &box[2]) &&
             next_items(r, b) && parse_int(b[0], natoms);
    } else if (a.size() == 1) {  // Natoms, then the box record
        ok = parse_int(a[0], natoms) && next_items(r, b) && b.size() >= 3 && parse_real(b[0], &box[0]) &&
             parse_real(b[1], &box[1]) && parse_real(b[2], &box[2]);
    }
    if (!ok || *natoms <= 0 || *natoms % 3) return PIMD_ERR_ARG;
    for (int c = 0; c < 3; c++)
        if (!(box[c] > 0) || !std::isfinite(box[c])) return PIMD_ERR_ARG;
    return PIMD_OK;
}

int pimd_read_xyz(const char *path, int read_method, int natoms, double *RRc) {
    if (!path || !RRc || natoms <= 0 || natoms % 3 || (read_method != 0 && read_method != 1)) return PIMD_ERR_ARG;
    int n = 0;
    double box[3];
    int rc = pimd_read_config_header(path, &n, nullptr, nullptr, box);
    if (rc) return rc;
    if (n != natoms || !ends_with(path, ".xyz")) return PIMD_ERR_ARG;
    // skip the header records again: they are the first one or two records with items
    LineReader r(path);
    std::vector<std::string> it;
    if (!next_items(r, it)) return PIMD_ERR_ARG;
    if (it.size() == 3 || it.size() == 1) {
        if (!next_items(r, it)) return PIMD_ERR_ARG;
    }
    const int N = natoms / 3;
    auto read_atom = [&](int i) {
        if (!next_items(r, it) || it.size() < 4) return false;
        for (int c = 0; c < 3; c++)
            if (!parse_real(it[1 + c], &RRc[3 * (size_t)i + c])) return false;
        return true;
    };
    double avg[3] = {0, 0, 0};
    if (read_method == 0) {
        for (int i = 0; i < N; i++)
            if (!read_atom(3 * i)) return PIMD_ERR_ARG;
        for (int i = 0; i < N; i++)
            if (!read_atom(3 * i + 1) || !read_atom(3 * i + 2)) return PIMD_ERR_ARG;
    } else {
        for (int i = 0; i < natoms; i++) {
            if (!read_atom(i)) return PIMD_ERR_ARG;
            for (int c = 0; c < 3; c++) avg[c] = avg[c] + RRc[3 * (size_t)i + c];
        }
    }
    for (int c = 0; c < 3; c++) avg[c] = avg[c] / natoms;
    for (int i = 0; i < natoms; i++)
        for (int c = 0; c < 3; c++) RRc[3 * (size_t)i + c] = RRc[3 * (size_t)i + c] - avg[c];
    return PIMD_OK;
}

int pimd_write_xyz(const char *path, int append, int natoms, const double *RR) {
    if (!path || !RR || natoms <= 0 || natoms % 3) return PIMD_ERR_ARG;
    FILE *f = std::fopen(path, append ? "a" : "w");
    if (!f) return PIMD_ERR_ARG;
    std::string out = write_i(natoms, 10) + "\n";
    out += " \n";  // write(iun,*) "": a list-directed record with one blank
    static const char *sym[3] = {"O ", "H ", "H "};
    for (int i = 0; i < natoms; i++) {
        out += sym[i % 3];
        for (int c = 0; c < 3; c++) out += " " + write_f(RR[3 * (size_t)i + c], 12, 6);
        out += "\n";
    }
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    return (std::fclose(f) == 0 && ok) ? PIMD_OK : PIMD_ERR_ARG;
}

int pimd_save_image(const char *path, int natoms, int nbeads, double time, const double *box, const double *RRt,
                    const double *PPt, double massO, double massH, const double *vxi_beads, int n_vxi_beads,
                    const double *vxi_global, int n_vxi_global) {
    if (!path || !box || !RRt || !PPt || natoms <= 0 || natoms % 3 || nbeads < 1 || !(massO > 0) || !(massH > 0))
        return PIMD_ERR_ARG;
    if ((n_vxi_beads && (!vxi_beads || n_vxi_beads != 2 * 3 * natoms * nbeads)) || (n_vxi_global && !vxi_global) ||
        n_vxi_beads < 0 || n_vxi_global < 0)
        return PIMD_ERR_ARG;
    FILE *f = std::fopen(path, "w");
    if (!f) return PIMD_ERR_ARG;
    std::string out = write_i(natoms, 10) + write_i(nbeads, 10) + "\n";
    out += write_f(time, 12, 6) + "  " + write_f(box[0], 12, 6);
    for (int c = 1; c < 3; c++) out += " " + write_f(box[c], 12, 6);
    out += "\n";
    const double imass[2] = {1.0 / massO, 1.0 / massH};  // imassO = DBLE(1/massO) (InputOutput.f90:135)
    const int N = natoms / 3;
    const size_t bs = (size_t)3 * natoms;
    for (int w = 0; w < N; w++)
        for (int a = 0; a < 3; a++) {
            const int i = 3 * w + a;
            for (int j = 0; j < nbeads; j++) {
                out += a == 0 ? "O " : "H ";
                for (int c = 0; c < 3; c++) out += " " + write_f(RRt[bs * j + 3 * (size_t)i + c], 12, 6);
                for (int c = 0; c < 3; c++)
                    out += " " + write_f(PPt[bs * j + 3 * (size_t)i + c] * imass[a == 0 ? 0 : 1], 12, 6);
                out += "\n";
            }
        }
    // vxi_beads(2, Natoms, Nbeads, 3): one record per (atom, bead, component), i fastest
    if (n_vxi_beads) {
        for (int i = 0; i < natoms; i++)
            for (int j = 0; j < nbeads; j++)
                for (int k = 0; k < 3; k++) {
                    const size_t o = 2 * ((size_t)i + (size_t)natoms * ((size_t)j + (size_t)nbeads * k));
                    out += write_ld(vxi_beads[o]) + write_ld(vxi_beads[o + 1]) + "\n";
                }
    }
    if (n_vxi_global) {
        for (int k = 0; k < n_vxi_global; k++) out += write_ld(vxi_global[k]);
        out += "\n";
    }
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    return (std::fclose(f) == 0 && ok) ? PIMD_OK : PIMD_ERR_ARG;
}

int pimd_load_image(const char *path, int natoms, int nbeads, double massO, double massH, double *time, double *box,
                    double *RRt, double *PPt, double *RRc, double *vxi_beads, int n_vxi_beads, double *vxi_global,
                    int n_vxi_global) {
    if (!path || !box || !RRt || !PPt || natoms <= 0 || natoms % 3 || nbeads < 1 || !(massO > 0) || !(massH > 0))
        return PIMD_ERR_ARG;
    if ((n_vxi_beads && (!vxi_beads || n_vxi_beads != 2 * 3 * natoms * nbeads)) || (n_vxi_global && !vxi_global) ||
        n_vxi_beads < 0 || n_vxi_global < 0)
        return PIMD_ERR_ARG;
    int n = 0, nb = 0;
    double tt = 0;
    int rc = pimd_read_config_header(path, &n, &nb, &tt, box);
    if (rc) return rc;
    if (n != natoms || nb != nbeads) return PIMD_ERR_ARG;  // InputOutput.f90:90-94
    if (time) *time = tt;
    LineReader r(path);
    r.next();
    r.next();
    const double mass[2] = {massO, massH};
    const int N = natoms / 3;
    const size_t bs = (size_t)3 * natoms;
    for (int w = 0; w < N; w++)
        for (int a = 0; a < 3; a++) {
            const int i = 3 * w + a;
            for (int j = 0; j < nbeads; j++) {
                if (!r.next()) return PIMD_ERR_ARG;
                double x[3], v[3];
                if (!read_image_atom(r.line, x, v)) return PIMD_ERR_ARG;
                for (int c = 0; c < 3; c++) {
                    RRt[bs * j + 3 * (size_t)i + c] = x[c];
                    PPt[bs * j + 3 * (size_t)i + c] = v[c] * mass[a == 0 ? 0 : 1];
                }
            }
        }
    std::vector<std::string> it;
    if (n_vxi_beads) {
        for (int i = 0; i < natoms; i++)
            for (int j = 0; j < nbeads; j++)
                for (int k = 0; k < 3; k++) {
                    const size_t o = 2 * ((size_t)i + (size_t)natoms * ((size_t)j + (size_t)nbeads * k));
                    if (!next_items(r, it) || it.size() < 2 || !parse_real(it[0], &vxi_beads[o]) ||
                        !parse_real(it[1], &vxi_beads[o + 1]))
                        return PIMD_ERR_ARG;
                }
    }
    if (n_vxi_global) {
        int got = 0;
        while (got < n_vxi_global) {
            if (!next_items(r, it)) return PIMD_ERR_ARG;
            for (size_t q = 0; q < it.size() && got < n_vxi_global; q++)
                if (!parse_real(it[q], &vxi_global[got++])) return PIMD_ERR_ARG;
        }
    }
    // RRc = sum(RRt,3)/Nbeads, then PBCs (main_stuff.f90:107-125, cubic: box(1) for every axis)
    std::vector<double> cen(bs, 0.0);
    for (int j = 0; j < nbeads; j++)
        for (size_t q = 0; q < bs; q++) cen[q] = cen[q] + RRt[bs * j + q];
    const double boxi0 = 1.0 / box[0];
    for (size_t q = 0; q < bs; q++) {
        const double c = cen[q] / nbeads;
        const double shift = box[0] * anint(c * boxi0);
        cen[q] = c - shift;
        for (int j = 0; j < nbeads; j++) RRt[bs * j + q] = RRt[bs * j + q] - shift;
    }
    if (RRc) std::memcpy(RRc, cen.data(), sizeof(double) * bs);
    return PIMD_OK;
}

}  // extern "C"

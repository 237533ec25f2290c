// drd_io.cpp — host-side file formats of the reference driver: the `input` deck read by
// list-directed READ (microfluidics_complex_domain/mcl6.f90:68-99) and the unformatted
// checkpoint records of inout.f90 and particles_move.f90:312-323.
//
// Fortran unformatted sequential files (gfortran and ifort defaults) frame each record with
// its byte length as a 4-byte little-endian integer before and after the data.  Records
// written by inout.f90 hold ((a(i,k),k=0,N),i=0,M): k fastest.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/drd_gb300.h"

namespace {

void set_err(char* err, int len, const std::string& msg) {
    if (!err || len <= 0) return;
    std::snprintf(err, (size_t)len, "%s", msg.c_str());
}

// First list-directed value of a record: leading blanks skipped, then a quoted string or a
// token ending at a blank, comma or slash.  Returns false for a record with no value (blank
// or starting with a slash terminator).
bool first_value(const std::string& line, std::string& out) {
    size_t i = 0;
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
    if (i >= line.size() || line[i] == '/') return false;
    if (line[i] == '\'' || line[i] == '"') {
        const char q = line[i++];
        out.clear();
        while (i < line.size()) {
            if (line[i] == q) {
                if (i + 1 < line.size() && line[i + 1] == q) {  // doubled quote
                    out.push_back(q);
                    i += 2;
                    continue;
                }
                break;
            }
            out.push_back(line[i++]);
        }
        return true;
    }
    size_t j = i;
    while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != ',' && line[j] != '/' && line[j] != '\r')
        ++j;
    out = line.substr(i, j - i);
    const size_t star = out.find('*');  // r*c repeat form: the value is c
    if (star != std::string::npos) out = out.substr(star + 1);
    return true;
}

bool parse_real(std::string s, double* v) {
    for (char& c : s)
        if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
    if (s.empty()) return false;
    char* end = nullptr;
    const double x = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') return false;
    *v = x;
    return true;
}

bool parse_int(const std::string& s, int32_t* v) {
    if (s.empty()) return false;
    char* end = nullptr;
    const long x = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end != '\0') return false;
    *v = (int32_t)x;
    return true;
}

bool write_record(FILE* f, const void* data, size_t bytes) {
    const uint32_t n = (uint32_t)bytes;
    return std::fwrite(&n, 4, 1, f) == 1 && (bytes == 0 || std::fwrite(data, 1, bytes, f) == bytes) &&
           std::fwrite(&n, 4, 1, f) == 1;
}

// Reads one record into `dst` (`bytes` expected; dst NULL skips it).  A record shorter than
// `bytes` fails; a longer one is read in part, as a Fortran READ of fewer items does.
bool read_record(FILE* f, void* dst, size_t bytes) {
    uint32_t n = 0, m = 0;
    if (std::fread(&n, 4, 1, f) != 1) return false;
    if (n < bytes) return false;
    if (dst && bytes && std::fread(dst, 1, bytes, f) != bytes) return false;
    if (std::fseek(f, (long)(n - (dst ? bytes : 0)), SEEK_CUR) != 0) return false;
    if (std::fread(&m, 4, 1, f) != 1) return false;
    return m == n;
}

long cidx(int nr, int i, int k) { return (long)(i + 1) + (long)(k + 1) * (nr + 2); }
long uidx(int nr, int i, int k) { return (long)(i + 1) + (long)(k + 1) * (nr + 3); }
long vidx(int nr, int i, int k) { return (long)(i + 1) + (long)k * (nr + 2); }

enum Shape { NODE, UF, VF, CELLS };
long at(Shape s, int nr, int i, int k) {
    switch (s) {
        case NODE: return (long)i + (long)k * (nr + 1);
        case UF: return uidx(nr, i, k);
        case VF: return vidx(nr, i, k);
        default: return cidx(nr, i, k);
    }
}

// ((a(i,k),k=0,nz),i=0,nr) gathered from / scattered to a Fortran-shaped array.
void gather(Shape s, int nr, int nz, const double* a, std::vector<double>& rec) {
    rec.resize((size_t)(nr + 1) * (nz + 1));
    size_t q = 0;
    for (int i = 0; i <= nr; ++i)
        for (int k = 0; k <= nz; ++k) rec[q++] = a[at(s, nr, i, k)];
}
void scatter(Shape s, int nr, int nz, const std::vector<double>& rec, double* a) {
    size_t q = 0;
    for (int i = 0; i <= nr; ++i)
        for (int k = 0; k <= nz; ++k) a[at(s, nr, i, k)] = rec[q++];
}

// Fortran E editing Ew.d with one leading zero digit (the default scale factor): the value as
// 0.d1d2...dd x 10^e, written in `w` columns right-justified; the exponent takes the form E+ee
// while |e| <= 99 and +eee without the letter up to 999 (Fortran 2018, 13.7.2.3.3).
std::string fortran_e(double x, int w, int d) {
    char buf[64];
    if (!std::isfinite(x)) {
        std::snprintf(buf, sizeof(buf), "%*s", w, std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
        return buf;
    }
    std::string mant;
    int e = 0;
    if (x != 0.0) {
        // d significant digits, rounded to nearest: "D.DDDDDDE+XX" -> mantissa digits and exponent
        std::snprintf(buf, sizeof(buf), "%.*E", d - 1, std::fabs(x));
        std::string t(buf);
        const size_t epos = t.find('E');
        for (size_t q = 0; q < epos; ++q)
            if (std::isdigit((unsigned char)t[q])) mant.push_back(t[q]);
        e = std::atoi(t.c_str() + epos + 1) + 1;
    } else {
        mant.assign((size_t)d, '0');
    }
    std::string out = (std::signbit(x) && x != 0.0) ? "-0." : "0.";
    out += mant;
    if (std::abs(e) <= 99) std::snprintf(buf, sizeof(buf), "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
    else std::snprintf(buf, sizeof(buf), "%c%03d", e < 0 ? '-' : '+', std::abs(e));
    out += buf;
    if ((int)out.size() < w) out.insert(0, (size_t)(w - (int)out.size()), ' ');
    if ((int)out.size() > w) out.assign((size_t)w, '*');
    return out;
}

int append_line(const char* path, const std::string& line) {
    FILE* f = std::fopen(path, "a");
    if (!f) return DRD_ERR_BADARG;
    const bool ok = std::fputs(line.c_str(), f) >= 0 && std::fputc('\n', f) != EOF;
    return (std::fclose(f) == 0 && ok) ? DRD_OK : DRD_ERR_BADARG;
}

}  // namespace

extern "C" {

int drd_write_fort23(const char* path, double t, const drd_diagnostics* d) {
    if (!path || !d) return DRD_ERR_BADARG;
    std::string line;
    for (double x : {t, d->e1, d->e2, d->e3, d->e4, d->dissip}) line += fortran_e(x, 14, 7);  // format 6e14.7
    return append_line(path, line);
}

int drd_write_fort22(const char* path, int kcount, double dt, const drd_diagnostics* d) {
    if (!path || !d) return DRD_ERR_BADARG;
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%12d", kcount);
    std::string line(buf);
    line += " " + fortran_e(dt * d->dissip, 24, 16) + " " + fortran_e(d->mass, 24, 16);
    return append_line(path, line);
}


int drd_read_deck(const char* path, drd_deck* deck, char* err, int err_len) {
    if (!path || !deck) {
        set_err(err, err_len, "null argument");
        return DRD_ERR_BADARG;
    }
    FILE* f = std::fopen(path, "r");
    if (!f) {
        set_err(err, err_len, std::string("cannot open ") + path);
        return DRD_ERR_BADARG;
    }
    std::memset(deck, 0, sizeof(*deck));
    // the READ list of mcl6.f90:69-100 in order: 'r' real, 'i' integer, 'c' character
    struct Item { char kind; void* dst; const char* name; };
    drd_deck& d = *deck;
    const Item items[] = {
        {'r', &d.xld, "xld"}, {'r', &d.re, "re"}, {'r', &d.ca, "ca"}, {'r', &d.vs, "vs"},
        {'r', &d.xlsT, "xlsT"}, {'r', &d.xlsB, "xlsB"}, {'r', &d.xlsL, "xlsL"}, {'r', &d.xlsR, "xlsR"},
        {'r', &d.uwT, "uwT"}, {'r', &d.uwB, "uwB"}, {'r', &d.slen, "slen"}, {'r', &d.shig, "shig"},
        {'r', &d.angle, "angle"}, {'r', &d.slipratio, "slipratio"}, {'i', &d.iflag, "iflag"},
        {'i', &d.istep, "istep"}, {'r', &d.tf, "tf"}, {'r', &d.I_thickness, "I_thickness"},
        {'r', &d.s_implicit, "s_implicit"}, {'r', &d.tol, "tol"}, {'r', &d.ggz, "ggz"}, {'r', &d.ggx, "ggx"},
        {'r', &d.time_step_change, "time_step_change"}, {'r', &d.lambda_rho, "lambda_rho"},
        {'r', &d.lambda_eta, "lambda_eta"}, {'r', &d.UU, "UU"}, {'c', &d.lr_bd_type, "lr_bd_type"},
        {'c', &d.top_type_ph, "top_type_ph"}, {'c', &d.bot_type_ph, "bot_type_ph"},
        {'c', &d.top_type_u, "top_type_u"}, {'c', &d.bot_type_u, "bot_type_u"},
        {'c', &d.is_complex_domain, "is_complex_domain"},
    };
    const int nitems = (int)(sizeof(items) / sizeof(items[0]));
    char buf[4096];
    int got = 0;
    int rc = DRD_OK;
    while (got < nitems && std::fgets(buf, sizeof(buf), f)) {
        std::string line(buf), val;
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
        if (!first_value(line, val)) continue;  // a record with no value: READ goes on to the next
        const Item& it = items[got];
        bool ok = true;
        if (it.kind == 'r') ok = parse_real(val, (double*)it.dst);
        else if (it.kind == 'i') ok = parse_int(val, (int32_t*)it.dst);
        else *(char*)it.dst = val.empty() ? ' ' : val[0];
        if (!ok) {
            set_err(err, err_len, std::string("bad value '") + val + "' for " + it.name);
            rc = DRD_ERR_BADARG;
            break;
        }
        ++got;
    }
    std::fclose(f);
    d.entries = got;
    if (rc == DRD_OK && got < 31) {
        set_err(err, err_len, "deck ends after " + std::to_string(got) + " values (31 needed)");
        rc = DRD_ERR_BADARG;
    }
    return rc;
}

int drd_params_from_deck(const drd_deck* d, int nr, int nz, int variant, drd_params* p) {
    if (!d || !p || nr < 3 || nz < 3 || !(d->slen > 0) || !(d->shig > 0)) return DRD_ERR_BADARG;
    std::memset(p, 0, sizeof(*p));
    p->nr = nr;
    p->nz = nz;
    p->variant = variant;
    p->precision = DRD_PREC_FP64;
    p->phi_mode = 1;
    p->lr_bd_type = (unsigned char)d->lr_bd_type;
    p->ch_maxit = 500;
    p->uv_maxit = 800;
    p->phmu_maxit = 5000;
    p->dr = d->slen / nr;                             // finit.f90:25
    p->dz = d->shig / nz;                             // finit.f90:26
    p->dt = std::fmin(p->dr, p->dz) * d->time_step_change;  // finit.f90:395-397
    p->xld = d->xld;
    p->re = d->re;
    p->ca = d->ca;
    p->I_thickness = d->I_thickness;
    p->s_implicit = d->s_implicit;
    p->tol = d->tol;
    p->ggx = d->ggx;
    p->ggz = d->ggz;
    p->uwT = d->uwT;
    p->uwB = d->uwB;
    p->UU = d->UU;
    p->twall = 0.1;                                   // mcl6.f90:140
    p->bdr_upp = 0.6725;                              // finit.f90:104-105
    p->bdr_low = 0.1725;
    p->angle = d->angle;
    p->xlsB = d->xlsB;
    p->penalty_k = 1.0E5;                             // global.f90:91
    p->lambda_rho = d->lambda_rho;
    p->lambda_eta = d->lambda_eta;
    p->bdr_ph_used_adjust = 1.0e-6;
    p->mixed_inner_tol = 0.2;
    p->mixed_max_refine = 30;
    p->uv_precond = DRD_UV_JACOBI;                    // PSolve_uv_2_CG of the MF application
    return DRD_OK;
}

int drd_output(const char* path, int nr, int nz, double dr, double dz, const double* x, const double* y,
               const double* u, const double* v, const double* p, const double* fa, const double* f2, double t) {
    if (!path || nr < 1 || nz < 1 || !u || !v || !p || !fa || !f2) return DRD_ERR_BADARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return DRD_ERR_BADARG;
    std::vector<double> rec, grid((size_t)(nr + 1) * (nz + 1));
    bool ok = true;
    for (int which = 0; which < 2 && ok; ++which) {
        const double* g = which ? y : x;
        if (!g) {  // r(i,k) = (i+0.5) dr, z(i,k) = (k+0.5) dz (finit.f90:34-35)
            for (int k = 0; k <= nz; ++k)
                for (int i = 0; i <= nr; ++i)
                    grid[(size_t)i + (size_t)k * (nr + 1)] = which ? (k + 0.5) * dz : (i + 0.5) * dr;
            g = grid.data();
        }
        gather(NODE, nr, nz, g, rec);
        ok = write_record(f, rec.data(), rec.size() * 8);
    }
    const struct { Shape s; const double* a; } fields[] = {{UF, u}, {VF, v}, {CELLS, p}, {CELLS, fa}, {CELLS, f2}};
    for (const auto& fl : fields) {
        if (!ok) break;
        gather(fl.s, nr, nz, fl.a, rec);
        ok = write_record(f, rec.data(), rec.size() * 8);
    }
    ok = ok && write_record(f, &t, 8);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? DRD_OK : DRD_ERR_BADARG;
}

int drd_input(const char* path, int nr, int nz, double* x, double* y, double* u, double* v, double* p, double* fa,
              double* t) {
    if (!path || nr < 1 || nz < 1) return DRD_ERR_BADARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return DRD_ERR_BADARG;
    std::vector<double> rec((size_t)(nr + 1) * (nz + 1));
    const size_t bytes = rec.size() * 8;
    const struct { Shape s; double* a; } fields[] = {{NODE, x}, {NODE, y}, {UF, u}, {VF, v}, {CELLS, p}, {CELLS, fa}};
    bool ok = true;
    for (const auto& fl : fields) {
        ok = read_record(f, fl.a ? rec.data() : nullptr, bytes);
        if (!ok) break;
        if (fl.a) scatter(fl.s, nr, nz, rec, fl.a);
    }
    double tv = 0.0;
    ok = ok && read_record(f, &tv, 8);  // the record after f: f2's in a file from output (inout.f90:56)
    std::fclose(f);
    if (!ok) return DRD_ERR_BADARG;
    if (t) *t = tv;
    return DRD_OK;
}

int drd_read_time(const char* path, int nr, int nz, double* t) {
    if (!path || !t || nr < 1 || nz < 1) return DRD_ERR_BADARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return DRD_ERR_BADARG;
    const size_t bytes = (size_t)(nr + 1) * (nz + 1) * 8;
    bool ok = true;
    for (int r = 0; r < 7 && ok; ++r) ok = read_record(f, nullptr, bytes);
    ok = ok && read_record(f, t, 8);
    std::fclose(f);
    return ok ? DRD_OK : DRD_ERR_BADARG;
}

int drd_output_particles(const char* path, int np, const double* points) {
    if (!path || np < 0 || (np > 0 && !points)) return DRD_ERR_BADARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return DRD_ERR_BADARG;
    bool ok = write_record(f, points, (size_t)np * 2 * 8);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? DRD_OK : DRD_ERR_BADARG;
}

}  // extern "C"

// hermes_io.cu -- text checkpoints in the format of the reference's writeQ /
// readQ (initialize.f90:474-565), host code only.
//
// File: one record per (basis b, variable v, k, j) -- b slowest, then v, k,
// j -- holding the nx values Q(1:nx, j, k, v, b); then one record
// "t dt nout mpi_nx mpi_ny mpi_nz".  The reference writes with list-directed
// output (compiler-dependent spacing and digits) and reads with list-directed
// input, so the reader here accepts what list-directed input accepts: values
// separated by blanks or commas, a record's values continued on following
// lines, repeat counts r*c and null values r*, D or E exponents or an exponent
// given by its sign alone (1.0-5), and a slash ending the list early.  The
// writer prints 17 significant digits (%.16E), which round-trip FP64 exactly
// and which a REAL*4 or REAL*8 list-directed read of the reference accepts.
// Rows are formatted on several host threads.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "hermes_gb300.h"

namespace {

constexpr int NQV = 11;

void set_err(char* err, size_t n, const std::string& m) {
    if (err && n) {
        std::strncpy(err, m.c_str(), n - 1);
        err[n - 1] = 0;
    }
}

bool dims_ok(int nx, int ny, int nz, int nb) {
    return nx > 0 && ny > 0 && nz > 0 && (nb == 4 || nb == 8 || nb == 10 || nb == 20 || nb == 27);
}

// ---- list-directed input ---------------------------------------------------
struct Reader {
    const char* p;
    const char* end;
    long line = 1;
    int repeat_left = 0;      // pending copies of a repeated value
    bool repeat_null = false;
    double repeat_val = 0.0;
    bool slash = false;       // a slash ended the current list

    void skip_blanks() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    }
    // start the next list at a new record
    void next_record() {
        repeat_left = 0;
        slash = false;
        while (p < end && *p != '\n') ++p;
        if (p < end) { ++p; ++line; }
    }
    // one token of the current list; false at end of file.  kind: 0 value, 1 null
    bool token(std::string& tok, int& kind) {
        for (;;) {
            skip_blanks();
            if (p >= end) return false;
            if (*p == '\n') { ++p; ++line; continue; }   // a list continues on the next record
            break;
        }
        if (*p == '/') { slash = true; ++p; return false; }
        if (*p == ',') { ++p; kind = 1; return true; }   // empty field: a null value
        const char* s = p;
        while (p < end && *p != ' ' && *p != '\t' && *p != '\r' && *p != '\n' && *p != ',' && *p != '/') ++p;
        tok.assign(s, p - s);
        skip_blanks();
        if (p < end && *p == ',') ++p;                   // the separator after a value
        kind = 0;
        return true;
    }
};

// a Fortran real constant: D/Q exponents, or an exponent given by its sign alone
bool parse_real(const std::string& t, double& v) {
    std::string s = t;
    for (auto& ch : s)
        if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'E';
    bool has_e = s.find_first_of("eE") != std::string::npos;
    if (!has_e) {
        for (size_t i = 1; i < s.size(); ++i)
            if ((s[i] == '+' || s[i] == '-') && (std::isdigit((unsigned char)s[i - 1]) || s[i - 1] == '.')) {
                s.insert(i, 1, 'E');
                break;
            }
    }
    errno = 0;
    char* e = nullptr;
    v = std::strtod(s.c_str(), &e);
    return e && *e == 0 && !s.empty();
}

// the next value of the current list: 1 value, 0 null (leave the target), -1 end of list/file, -2 bad token
int next_value(Reader& r, double& v, std::string& bad) {
    if (r.slash) return -1;
    if (r.repeat_left > 0) {
        --r.repeat_left;
        if (r.repeat_null) return 0;
        v = r.repeat_val;
        return 1;
    }
    // fast path: a plain number followed by a separator
    for (;;) {
        r.skip_blanks();
        if (r.p < r.end && *r.p == '\n') { ++r.p; ++r.line; continue; }
        break;
    }
    if (r.p < r.end && *r.p != ',' && *r.p != '/') {
        char* e = nullptr;
        const double x = std::strtod(r.p, &e);
        if (e != r.p && e <= r.end &&
            (e == r.end || *e == ' ' || *e == '\t' || *e == '\r' || *e == '\n' || *e == ',' || *e == '/')) {
            r.p = e;
            r.skip_blanks();
            if (r.p < r.end && *r.p == ',') ++r.p;
            v = x;
            return 1;
        }
    }
    std::string tok;
    int kind = 0;
    if (!r.token(tok, kind)) return -1;
    if (kind == 1) return 0;
    const size_t star = tok.find('*');
    if (star != std::string::npos) {
        char* e = nullptr;
        const long n = std::strtol(tok.substr(0, star).c_str(), &e, 10);
        if (!e || *e != 0 || n < 1) { bad = tok; return -2; }
        const std::string rest = tok.substr(star + 1);
        r.repeat_null = rest.empty();
        if (!r.repeat_null && !parse_real(rest, r.repeat_val)) { bad = tok; return -2; }
        r.repeat_left = (int)n - 1;
        if (r.repeat_null) return 0;
        v = r.repeat_val;
        return 1;
    }
    if (!parse_real(tok, v)) { bad = tok; return -2; }
    return 1;
}

}  // namespace

extern "C" {

int hermes_checkpoint_write(const char* path, const double* q, int32_t nx, int32_t ny, int32_t nz, int32_t nbasis,
                            double t, double dt, int32_t nout, const int32_t* mpi_dims, char* err, size_t errlen) {
    if (!path || !q) { set_err(err, errlen, "null argument"); return HERMES_ERR_ARG; }
    if (!dims_ok(nx, ny, nz, nbasis)) { set_err(err, errlen, "bad grid dimensions or nbasis"); return HERMES_ERR_SHAPE; }
    const long long rows = (long long)nbasis * NQV * nz * ny;
    unsigned nth = std::thread::hardware_concurrency();
    if (nth < 1) nth = 1;
    if (nth > 32) nth = 32;
    if ((long long)nth > rows) nth = (unsigned)rows;
    std::vector<std::string> parts(nth);
    auto work = [&](unsigned w) {
        const long long r0 = rows * w / nth, r1 = rows * (w + 1) / nth;
        std::string& out = parts[w];
        out.reserve((size_t)((r1 - r0) * (nx * 24 + 2)));
        char buf[40];
        for (long long r = r0; r < r1; ++r) {
            const double* row = q + r * nx;   // (b, v, k, j) rows are contiguous in x
            for (int i = 0; i < nx; ++i) {
                const int n = std::snprintf(buf, sizeof buf, " %.16E", row[i]);
                out.append(buf, (size_t)n);
            }
            out.push_back('\n');
        }
    };
    std::vector<std::thread> th;
    for (unsigned w = 1; w < nth; ++w) th.emplace_back(work, w);
    work(0);
    for (auto& x : th) x.join();
    FILE* f = std::fopen(path, "wb");
    if (!f) { set_err(err, errlen, std::string("cannot open ") + path + ": " + std::strerror(errno)); return HERMES_ERR_ARG; }
    bool ok = true;
    for (auto& s : parts) ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
    const int md[3] = {mpi_dims ? mpi_dims[0] : 1, mpi_dims ? mpi_dims[1] : 1, mpi_dims ? mpi_dims[2] : 1};
    ok = ok && std::fprintf(f, " %.16E %.16E %d %d %d %d\n", t, dt, nout, md[0], md[1], md[2]) > 0;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { set_err(err, errlen, std::string("write failed: ") + path); return HERMES_ERR_ARG; }
    return HERMES_OK;
}

int hermes_checkpoint_read(const char* path, double* q, int32_t nx, int32_t ny, int32_t nz, int32_t nbasis,
                           double* t, double* dt, int32_t* nout, int32_t* mpi_dims, char* err, size_t errlen) {
    if (!path || !q) { set_err(err, errlen, "null argument"); return HERMES_ERR_ARG; }
    if (!dims_ok(nx, ny, nz, nbasis)) { set_err(err, errlen, "bad grid dimensions or nbasis"); return HERMES_ERR_SHAPE; }
    FILE* f = std::fopen(path, "rb");
    if (!f) { set_err(err, errlen, std::string("cannot open ") + path + ": " + std::strerror(errno)); return HERMES_ERR_ARG; }
    std::string buf;
    char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.append(chunk, n);
    std::fclose(f);
    Reader r{buf.data(), buf.data() + buf.size()};
    const long long rows = (long long)nbasis * NQV * nz * ny;
    std::string bad;
    for (long long row = 0; row < rows; ++row) {
        double* dst = q + row * nx;
        for (int i = 0; i < nx; ++i) {
            double v;
            const int k = next_value(r, v, bad);
            if (k == -2) {
                set_err(err, errlen, "bad value '" + bad + "' at line " + std::to_string(r.line));
                return HERMES_ERR_SHAPE;
            }
            if (k == -1) {
                if (r.slash) break;   // the rest of this list keeps its previous values
                set_err(err, errlen, "file ends in record " + std::to_string(row + 1) + " of " + std::to_string(rows));
                return HERMES_ERR_SHAPE;
            }
            if (k == 1) dst[i] = v;
        }
        r.next_record();
    }
    double tail[6] = {t ? *t : 0.0, dt ? *dt : 0.0, (double)(nout ? *nout : 0), (double)(mpi_dims ? mpi_dims[0] : 1),
                      (double)(mpi_dims ? mpi_dims[1] : 1), (double)(mpi_dims ? mpi_dims[2] : 1)};
    for (int i = 0; i < 6; ++i) {
        double v;
        const int k = next_value(r, v, bad);
        if (k == -2) { set_err(err, errlen, "bad value '" + bad + "' in the last record"); return HERMES_ERR_SHAPE; }
        if (k == -1) {
            if (r.slash) break;
            set_err(err, errlen, "the last record (t dt nout mpi_nx mpi_ny mpi_nz) is incomplete");
            return HERMES_ERR_SHAPE;
        }
        if (k == 1) tail[i] = v;
    }
    if (t) *t = tail[0];
    if (dt) *dt = tail[1];
    if (nout) *nout = (int32_t)std::llround(tail[2]);
    if (mpi_dims)
        for (int i = 0; i < 3; ++i) mpi_dims[i] = (int32_t)std::llround(tail[3 + i]);
    return HERMES_OK;
}

}  // extern "C"

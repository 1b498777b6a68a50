// grid_io.cpp -- reader of PLES's grid file gri3dp_in.dat (host code only).
//
// The file is what fsrc/stratiParticle.f03:364-412 reads with Fortran
// list-directed input: a record with the domain lengths alx aly alz, a
// record with the cell counts jx jy jz, then for every node (i fastest, then
// j, then k) three records holding x, y and z.  A list-directed READ of one
// variable starts at a new record and takes its first value, so anything
// after the first value of a coordinate record is ignored; the header READs
// take their values from as many records as they need.  Fortran exponent
// letters D/d and Q/q are read as E.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ples_mg.h"

namespace {

struct Records {
    FILE* f = nullptr;
    std::vector<char> line;
    ~Records() {
        if (f) std::fclose(f);
    }
    // next record into line (without its terminator); false at end of file
    bool next() {
        line.clear();
        int ch;
        bool any = false;
        while ((ch = std::fgetc(f)) != EOF) {
            any = true;
            if (ch == '\n') break;
            line.push_back((char)ch);
        }
        if (!any) return false;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        line.push_back('\0');
        return true;
    }
};

// list-directed separators: blanks, tabs, commas
bool is_sep(char c) { return c == ' ' || c == '\t' || c == ','; }

// parse one value token at *s; advances *s past it
bool parse_double(const char** s, double* out) {
    const char* p = *s;
    while (*p && is_sep(*p)) ++p;
    if (!*p) return false;
    char tok[128];
    int n = 0;
    while (p[n] && !is_sep(p[n]) && p[n] != '/') {
        if (n >= (int)sizeof tok - 1) return false;
        char c = p[n];
        if (c == 'D' || c == 'd' || c == 'Q' || c == 'q') c = 'E';
        tok[n++] = c;
    }
    tok[n] = '\0';
    if (n == 0) return false;
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(tok, &end);
    if (end != tok + n || errno == ERANGE) return false;
    *out = v;
    *s = p + n;
    return true;
}

// one list-directed READ of cnt values starting at a new record
bool read_values(Records& r, int cnt, double* out) {
    int got = 0;
    while (got < cnt) {
        if (!r.next()) return false;
        const char* s = r.line.data();
        while (got < cnt && parse_double(&s, &out[got])) ++got;
    }
    return true;
}

}  // namespace

extern "C" int ples_mg_read_grid(const char* path, double lengths[3], int dims[3], double* x, double* y, double* z) {
    if (!path || !dims) return PLES_MG_BAD_ARG;
    Records r;
    r.f = std::fopen(path, "rb");
    if (!r.f) return PLES_MG_BAD_ARG;
    double len[3], nd[3];
    if (!read_values(r, 3, len) || !read_values(r, 3, nd)) return PLES_MG_BAD_ARG;
    int n[3];
    for (int c = 0; c < 3; ++c) {
        if (!(nd[c] >= 1.0 && nd[c] <= 1e6) || nd[c] != (double)(int)nd[c]) return PLES_MG_BAD_ARG;
        n[c] = (int)nd[c];
        dims[c] = n[c];
        if (lengths) lengths[c] = len[c];
    }
    if (!x && !y && !z) return PLES_MG_OK;  // sizes only
    if (!x || !y || !z) return PLES_MG_BAD_ARG;
    const long long nodes = (long long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
    double* dst[3] = {x, y, z};
    for (long long q = 0; q < nodes; ++q)
        for (int c = 0; c < 3; ++c)
            if (!read_values(r, 1, &dst[c][q])) return PLES_MG_BAD_ARG;
    return PLES_MG_OK;
}

// PHASTA's POSIX file format and the compressible solver's mesh/restart I/O on the host.
//
// Format (phastaIO/phastaIO.cc, POSIX branch): a file is a sequence of text header lines
// "key : < n > i1 i2 ... \n", each followed by n bytes of data (binary: the values and one
// '\n'; ascii: n lines of one value).  Text after '#' and empty lines are comments.  A
// reader searches the header of a key from its current position, skipping the data of
// other headers by their byte counts, and wraps around to the start of the file once.
// The block "byteorder magic number" holds the integer 362436; a reader that meets it with
// another value swaps the bytes of every later block.
//
// The geombc reader follows readnblk.f:112-385 (single rank), genblkPosix.f and
// genbkbPosix.f; the restart reader/writer readnblk.f:480-545, restar.f and
// new_interface.c:240-330; geniBC/genBC1 the reference's genibc.f and genbc1.f.

#include "../../include/phgpu_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <dirent.h>
#include <iterator>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

namespace {

constexpr int kMagic = 362436;  // phastaIO.cc:256
constexpr int kLine = 1024;     // header lines are read in pieces of at most 1023 characters

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

// Key comparison of phastaIO (cscompare, phastaIO.cc:179-195): blanks are skipped on both
// sides, letters compare without case, a '?' in the file's key or the end of `phrase` ends
// the comparison; `phrase` matches when it is used up or reaches a '?'.
bool key_match(const char* phrase, const char* token) {
    auto blanks = [](const char*& p) {
        while (*p == ' ') ++p;
    };
    const char* a = phrase;
    const char* b = token;
    blanks(a);
    blanks(b);
    while (*a && *b && *b != '?' &&
           std::tolower((unsigned char)*a) == std::tolower((unsigned char)*b)) {
        ++a;
        ++b;
        blanks(a);
        blanks(b);
    }
    return *a == 0 || *a == '?';
}

// the part of a type or mode string before its first blank (StringStripper, :168-176)
std::string first_word(const char* s) {
    std::string r(s ? s : "");
    size_t sp = r.find(' ');
    if (sp != std::string::npos) r.resize(sp);
    return r;
}

bool is_binary(const char* iotype) { return key_match(first_word(iotype).c_str(), "binary"); }

size_t type_size(const char* datatype) {
    std::string t = first_word(datatype);
    if (key_match("integer", t.c_str())) return sizeof(int32_t);
    if (key_match("double", t.c_str())) return sizeof(double);
    return 0;
}

// Tokens of a header line after its key: separated by any of " ,;<>" (the newline is
// not a separator, as in the reference, so a trailing "\n" is a token of value 0)
std::vector<std::string> split_fields(const std::string& s) {
    std::vector<std::string> out;
    size_t i = 0;
    const char* sep = " ,;<>";
    while (i < s.size()) {
        while (i < s.size() && std::strchr(sep, s[i])) ++i;
        if (i >= s.size()) break;
        size_t j = i;
        while (j < s.size() && !std::strchr(sep, s[j])) ++j;
        out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

void swap_bytes(void* p, size_t size, size_t n) {
    unsigned char* c = (unsigned char*)p;
    for (size_t k = 0; k < n; ++k, c += size)
        for (size_t j = 0; j < size / 2; ++j) std::swap(c[j], c[size - 1 - j]);
}

struct PhFile {
    FILE* f = nullptr;
    bool swap = false;             // byte order of the data differs from this machine's
    std::string last_key;          // key of the header read or written last ("" after its block)
    bool last_not_found = false;   // the last header search failed
    size_t header_type = sizeof(int32_t);
    long long data_items = 0;      // items announced by the last header written
};

std::mutex g_mu;
std::vector<std::unique_ptr<PhFile>> g_files;  // descriptor d is g_files[d - 1]; never reused
bool g_strict = false;

PhFile* get(int fd) {
    if (fd < 1 || fd > (int)g_files.size() || !g_files[fd - 1]) return nullptr;
    return g_files[fd - 1].get();
}

bool next_line(PhFile& F, char* line, int& rewinds) {
    if (std::fgets(line, kLine, F.f)) return true;
    if (!std::feof(F.f)) return false;
    std::rewind(F.f);
    std::clearerr(F.f);
    ++rewinds;
    if (!std::fgets(line, kLine, F.f)) line[0] = 0;
    return true;
}

int search_header_from(PhFile& F, const char* phrase, int* params, int expect, bool binary) {
    char line[kLine] = "";
    int rewinds = 0;
    if (!next_line(F, line, rewinds)) return -1;
    bool found = false;
    while (!found && rewinds < 2) {
        size_t len = std::strcspn(line, "#");
        if (line[0] != '\n' && line[0] != 0 && len > 0) {
            std::string text(line, len);
            // the key is the text up to the first ':' (leading ':' skipped, as strtok does)
            size_t k0 = text.find_first_not_of(':');
            if (k0 == std::string::npos) return -1;
            size_t k1 = text.find(':', k0);
            std::string key = text.substr(k0, k1 == std::string::npos ? std::string::npos : k1 - k0);
            std::string rest = k1 == std::string::npos ? std::string() : text.substr(k1 + 1);
            std::vector<std::string> f = split_fields(rest);
            if (key_match(phrase, key.c_str())) {
                found = true;
                if (f.empty()) return -1;
                int i = 0;
                for (; i < expect && i + 1 < (int)f.size(); ++i) params[i] = std::atoi(f[i + 1].c_str());
                (void)i;
            } else if (key_match(key.c_str(), "byteorder magic number")) {
                int v = 0;
                if (binary) {
                    char junk;
                    if (std::fread(&v, sizeof v, 1, F.f) != 1) return -1;
                    if (std::fread(&junk, 1, 1, F.f) != 1) return -1;
                    if (v != kMagic) F.swap = true;
                } else if (std::fscanf(F.f, "%d\n", &v) != 1) {
                    return -1;
                }
            } else {
                if (f.empty()) return -1;
                long skip = std::atol(f[0].c_str());
                if (binary) {
                    if (std::fseek(F.f, skip, SEEK_CUR) != 0) return -1;
                } else {
                    for (long g = 0; g < skip; ++g)
                        if (!std::fgets(line, kLine, F.f)) break;
                }
            }
        }
        if (!found && !next_line(F, line, rewinds)) return -1;
    }
    return found ? 0 : 1;
}

// readHeader (phastaIO.cc:197-306): 0 found, 1 not found, -1 malformed file.  A failed
// search puts the file back where it started; the reference leaves it after the first
// header line, so that its next search reads the magic number's data as a header line and
// stops on an assert there (phastaIO.cc:279).
int search_header(PhFile& F, const char* phrase, int* params, int expect, bool binary) {
    const long start = std::ftell(F.f);
    int r = search_header_from(F, phrase, params, expect, binary);
    if (r == 1 && start >= 0) {
        std::clearerr(F.f);
        std::fseek(F.f, start, SEEK_SET);
    }
    return r;
}

std::string part_name(const char* dir, const std::string& base, int rank) {
    std::string d(dir ? dir : ".");
    if (!d.empty() && d.back() != '/') d += '/';
    return d + base + std::to_string(rank + 1);
}

// one open file, closed on scope exit
struct Open {
    int fd = 0;
    std::string mode;
    Open(const std::string& name, const char* m) : mode(m) {
        if (phgpu_io_openfile(name.c_str(), m, &fd) != PHGPU_OK) fd = 0;
    }
    ~Open() {
        if (fd) phgpu_io_closefile(fd, mode.c_str());
    }
};

}  // namespace

extern "C" {

const char* phgpu_io_last_error(void) { return g_err.c_str(); }

int phgpu_io_togglestrictmode(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_strict = !g_strict;
    return g_strict ? 1 : 0;
}

int phgpu_io_openfile(const char* filename, const char* mode, int* fd) {
    if (!filename || !mode || !fd) return fail(PHGPU_ERR_INVALID, "openfile: null argument");
    *fd = 0;
    std::string m = first_word(mode), name = first_word(filename);
    const char* cm = key_match("read", m.c_str())     ? "rb"
                     : key_match("write", m.c_str())  ? "wb"
                     : key_match("append", m.c_str()) ? "ab"
                                                      : nullptr;
    if (!cm) return fail(PHGPU_ERR_INVALID, "openfile: unknown mode '%s'", mode);
    FILE* f = std::fopen(name.c_str(), cm);
    if (!f) return fail(PHGPU_ERR_IO, "openfile: unable to open file %s", name.c_str());
    std::lock_guard<std::mutex> lk(g_mu);
    g_files.emplace_back(new PhFile);
    g_files.back()->f = f;
    *fd = (int)g_files.size();
    return PHGPU_OK;
}

int phgpu_io_closefile(int fd, const char* mode) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F) return fail(PHGPU_ERR_INVALID, "closefile: no file associated with descriptor %d", fd);
    std::string m = first_word(mode);
    int rc = PHGPU_OK;
    if ((key_match("write", m.c_str()) || key_match("append", m.c_str())) && std::fflush(F->f) != 0)
        rc = fail(PHGPU_ERR_IO, "closefile: flush failed");
    if (std::fclose(F->f) != 0 && rc == PHGPU_OK) rc = fail(PHGPU_ERR_IO, "closefile: close failed");
    g_files[fd - 1].reset();
    return rc;
}

int phgpu_io_readheader(int fd, const char* keyphrase, int* values, int nitems, const char* datatype,
                        const char* iotype) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F) return fail(PHGPU_ERR_INVALID, "readheader: no file associated with descriptor %d", fd);
    if (!keyphrase || (nitems > 0 && !values) || nitems < 0) return fail(PHGPU_ERR_INVALID, "readheader: bad argument");
    F->last_key = keyphrase;
    F->last_not_found = false;
    (void)datatype;
    int r = search_header(*F, keyphrase, values, nitems, is_binary(iotype));
    if (r < 0) {
        F->last_not_found = true;
        return fail(PHGPU_ERR_IO, "readheader: malformed or unreadable file while searching '%s'", keyphrase);
    }
    if (r > 0) {
        F->last_not_found = true;
        return fail(PHGPU_ERR_NOTFOUND, "readheader: could not find '%s'", keyphrase);
    }
    return PHGPU_OK;
}

int phgpu_io_readdatablock(int fd, const char* keyphrase, void* values, int nitems, const char* datatype,
                           const char* iotype) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F) return fail(PHGPU_ERR_INVALID, "readdatablock: no file associated with descriptor %d", fd);
    if (!keyphrase || nitems < 0 || (nitems > 0 && !values)) return fail(PHGPU_ERR_INVALID, "readdatablock: bad argument");
    if (!key_match(F->last_key.c_str(), keyphrase) && g_strict)
        return fail(PHGPU_ERR_IO, "readdatablock: header '%s' not consistent with data block '%s'",
                    F->last_key.c_str(), keyphrase);
    if (F->last_not_found) return fail(PHGPU_ERR_NOTFOUND, "readdatablock: header of '%s' was not found", keyphrase);
    F->last_key.clear();
    size_t ts = type_size(datatype);
    if (!ts) return fail(PHGPU_ERR_INVALID, "readdatablock: unknown type '%s'", datatype ? datatype : "");
    if (is_binary(iotype)) {
        if (std::fread(values, ts, (size_t)nitems, F->f) != (size_t)nitems)
            return fail(PHGPU_ERR_IO, "readdatablock: short read of '%s'", keyphrase);
        char junk;
        if (std::fread(&junk, 1, 1, F->f) != 1 && nitems > 0)
            return fail(PHGPU_ERR_IO, "readdatablock: missing end of block '%s'", keyphrase);
        if (F->swap) swap_bytes(values, ts, (size_t)nitems);
    } else if (ts == sizeof(int32_t)) {
        for (int n = 0; n < nitems; ++n)
            if (std::fscanf(F->f, "%d\n", (int*)values + n) != 1)
                return fail(PHGPU_ERR_IO, "readdatablock: bad integer in '%s'", keyphrase);
    } else {
        for (int n = 0; n < nitems; ++n)
            if (std::fscanf(F->f, "%lf\n", (double*)values + n) != 1)
                return fail(PHGPU_ERR_IO, "readdatablock: bad value in '%s'", keyphrase);
    }
    return PHGPU_OK;
}

int phgpu_io_writeheader(int fd, const char* keyphrase, const int* values, int nitems, int ndataitems,
                         const char* datatype, const char* iotype) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F) return fail(PHGPU_ERR_INVALID, "writeheader: no file associated with descriptor %d", fd);
    if (!keyphrase || nitems < 0 || ndataitems < 0 || (nitems > 0 && !values))
        return fail(PHGPU_ERR_INVALID, "writeheader: bad argument");
    size_t ts = type_size(datatype);
    F->last_key = keyphrase;
    F->data_items = ndataitems;
    F->header_type = ts;
    long long bytes = is_binary(iotype) ? (long long)ts * ndataitems + (ndataitems > 0 ? 1 : 0) : ndataitems;
    if (bytes > INT_MAX) return fail(PHGPU_ERR_TOO_LARGE, "writeheader: block '%s' of %lld bytes", keyphrase, bytes);
    if (std::fprintf(F->f, "%s : < %d > ", keyphrase, (int)bytes) < 0) return fail(PHGPU_ERR_IO, "writeheader: write failed");
    for (int i = 0; i < nitems; ++i) std::fprintf(F->f, "%d ", values[i]);
    if (std::fprintf(F->f, "\n") < 0) return fail(PHGPU_ERR_IO, "writeheader: write failed");
    return PHGPU_OK;
}

int phgpu_io_writedatablock(int fd, const char* keyphrase, const void* values, int nitems,
                            const char* datatype, const char* iotype) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F) return fail(PHGPU_ERR_INVALID, "writedatablock: no file associated with descriptor %d", fd);
    if (!keyphrase || nitems < 0 || (nitems > 0 && !values)) return fail(PHGPU_ERR_INVALID, "writedatablock: bad argument");
    if (!key_match(F->last_key.c_str(), keyphrase) && g_strict)
        return fail(PHGPU_ERR_IO, "writedatablock: header '%s' not consistent with data block '%s'",
                    F->last_key.c_str(), keyphrase);
    size_t ts = type_size(datatype);
    if (!ts) return fail(PHGPU_ERR_INVALID, "writedatablock: unknown type '%s'", datatype ? datatype : "");
    F->last_key.clear();
    if (g_strict && (F->header_type != ts || F->data_items != nitems))
        return fail(PHGPU_ERR_IO, "writedatablock: header and data block of '%s' differ", keyphrase);
    if (is_binary(iotype)) {
        if (std::fwrite(values, ts, (size_t)nitems, F->f) != (size_t)nitems || std::fprintf(F->f, "\n") < 0)
            return fail(PHGPU_ERR_IO, "writedatablock: write of '%s' failed", keyphrase);
    } else if (ts == sizeof(int32_t)) {
        for (int n = 0; n < nitems; ++n) std::fprintf(F->f, "%d\n", ((const int*)values)[n]);
    } else {
        for (int n = 0; n < nitems; ++n) std::fprintf(F->f, "%f\n", ((const double*)values)[n]);
    }
    return PHGPU_OK;
}

int phgpu_io_writestring(int fd, const char* text) {
    std::lock_guard<std::mutex> lk(g_mu);
    PhFile* F = get(fd);
    if (!F || !text) return fail(PHGPU_ERR_INVALID, "writestring: bad argument");
    return std::fputs(text, F->f) < 0 ? fail(PHGPU_ERR_IO, "writestring: write failed") : PHGPU_OK;
}

// ---- restart files ----------------------------------------------------------------------

// file order (p, u, v, w, T, ...) <-> solver order (u, v, w, p, T, ...) (restar.f:40-48, 70-78)
static void to_file_order(const double* y, double* q, size_t nshg, int ndof) {
    std::memcpy(q, y + 3 * nshg, sizeof(double) * nshg);
    std::memcpy(q + nshg, y, sizeof(double) * 3 * nshg);
    if (ndof > 4) std::memcpy(q + 4 * nshg, y + 4 * nshg, sizeof(double) * (ndof - 4) * nshg);
}

static void to_solver_order(const double* q, double* y, size_t nshg, int ndof) {
    std::memcpy(y, q + nshg, sizeof(double) * 3 * nshg);
    std::memcpy(y + 3 * nshg, q, sizeof(double) * nshg);
    if (ndof > 4) std::memcpy(y + 4 * nshg, q + 4 * nshg, sizeof(double) * (ndof - 4) * nshg);
}

int phgpu_io_write_restart(const char* dir, int rank, int stepno, int nshg, int ndof, const double* y,
                           const double* ac) {
    if (nshg <= 0 || ndof < 4 || !y || !ac || rank < 0) return fail(PHGPU_ERR_INVALID, "write_restart: bad argument");
    if ((long long)nshg * ndof * 8 + 1 > INT_MAX) return fail(PHGPU_ERR_TOO_LARGE, "write_restart: field too large");
    std::string name = part_name(dir, "restart." + std::to_string(stepno) + ".", rank);
    Open o(name, "write");
    if (!o.fd) return fail(PHGPU_ERR_IO, "write_restart: unable to open %s", name.c_str());
    const char* mkey = "byteorder magic number";
    int magic = kMagic, one = 1;
    int rc = phgpu_io_writeheader(o.fd, mkey, &magic, 1, 1, "integer", "binary");
    if (!rc) rc = phgpu_io_writedatablock(o.fd, mkey, &magic, one, "integer", "binary");
    std::vector<double> q((size_t)nshg * ndof);
    const int isize = nshg * ndof;
    int head[3] = {nshg, ndof, stepno};
    const char* keys[2] = {"solution", "time derivative of solution"};
    const double* src[2] = {y, ac};
    for (int k = 0; k < 2 && !rc; ++k) {
        to_file_order(src[k], q.data(), nshg, ndof);
        rc = phgpu_io_writeheader(o.fd, keys[k], head, 3, isize, "double", "binary");
        if (!rc) rc = phgpu_io_writedatablock(o.fd, keys[k], q.data(), isize, "double", "binary");
    }
    return rc;
}

int phgpu_io_read_restart(const char* dir, int rank, int irstart, int nshg, int ndof, double* y, double* ac,
                          int* lstep) {
    if (nshg <= 0 || ndof < 4 || !y || !ac || rank < 0) return fail(PHGPU_ERR_INVALID, "read_restart: bad argument");
    std::string name = part_name(dir, "restart." + std::to_string(irstart) + ".", rank);
    Open o(name, "read");
    if (!o.fd) return fail(PHGPU_ERR_IO, "read_restart: unable to open %s", name.c_str());
    const char* keys[2] = {"solution", "time derivative of solution"};
    double* dst[2] = {y, ac};
    std::vector<double> q((size_t)nshg * ndof), buf;
    int step = 0;
    for (int k = 0; k < 2; ++k) {
        int head[3] = {0, 0, 0};
        int rc = phgpu_io_readheader(o.fd, keys[k], head, 3, "integer", "binary");
        if (rc != PHGPU_OK && rc != PHGPU_ERR_NOTFOUND) return rc;
        if (rc == PHGPU_OK && head[0] != 0) {
            if (head[0] != nshg) return fail(PHGPU_ERR_INVALID, "read_restart: '%s' has nshg %d, expected %d", keys[k], head[0], nshg);
            if (head[1] < ndof) return fail(PHGPU_ERR_INVALID, "read_restart: '%s' has %d dofs, expected %d", keys[k], head[1], ndof);
            step = head[2];
            buf.assign((size_t)head[0] * head[1], 0.0);
            rc = phgpu_io_readdatablock(o.fd, keys[k], buf.data(), head[0] * head[1], "double", "binary");
            if (rc) return rc;
            std::copy(buf.begin(), buf.begin() + (size_t)nshg * ndof, q.begin());
        } else {
            // the compressible solver starts from p = T = 1 and a zero time derivative
            std::fill(q.begin(), q.end(), 0.0);
            if (k == 0) {
                std::fill(q.begin(), q.begin() + nshg, 1.0);
                std::fill(q.begin() + 4 * (size_t)nshg, q.begin() + 5 * (size_t)nshg, 1.0);
            }
        }
        to_solver_order(q.data(), dst[k], nshg, ndof);
    }
    if (lstep) *lstep = step;
    return PHGPU_OK;
}

// ---- geombc -----------------------------------------------------------------------------

struct phgpu_geombc {
    phgpu_geombc_info info{};
    std::vector<double> x, BCinp;
    std::vector<int> nBC, iBCtmp, iper;
    std::vector<phgpu_topblock> interior, boundary;
    std::vector<std::vector<int>> ien, ienb, iBCB;
    std::vector<std::vector<double>> BCB;
    int ndof = 5;
};

static int read_int_header(int fd, const char* key, int* v, int n) {
    return phgpu_io_readheader(fd, key, v, n, "integer", "binary");
}

int phgpu_io_geombc_open(const char* dir, int rank, int ndof, phgpu_geombc** out) {
    if (!out || rank < 0 || ndof < 5) return fail(PHGPU_ERR_INVALID, "geombc_open: bad argument");
    *out = nullptr;
    std::string name = part_name(dir, "geombc.dat.", rank);
    Open o(name, "read");
    if (!o.fd) return fail(PHGPU_ERR_IO, "geombc_open: unable to open %s", name.c_str());
    std::unique_ptr<phgpu_geombc> g(new phgpu_geombc);
    g->ndof = ndof;
    phgpu_geombc_info& I = g->info;
    struct {
        const char* key;
        int* dst;
    } counts[] = {{"number of nodes", &I.numnp},
                  {"number of modes", &I.nshg},
                  {"number of interior elements", &I.numel},
                  {"number of boundary elements", &I.numelb},
                  {"maximum number of element nodes", &I.nen},
                  {"number of interior tpblocks", &I.nelblk},
                  {"number of boundary tpblocks", &I.nelblb},
                  {"number of nodes with Dirichlet BCs", &I.numpbc},
                  {"number of shape functions", &I.ntopsh}};
    for (auto& c : counts) {
        int rc = read_int_header(o.fd, c.key, c.dst, 1);
        if (rc) return rc;
    }
    int two[2] = {0, 0};
    int rc = phgpu_io_readheader(o.fd, "co-ordinates", two, 2, "double", "binary");
    if (rc) return rc;
    I.numnp = two[0];
    I.nsd = two[1];
    if (I.numnp <= 0 || I.nsd != 3 || I.nshg <= 0 || I.nelblk < 0 || I.nelblb < 0 || I.numpbc < 0)
        return fail(PHGPU_ERR_INVALID, "geombc_open: bad counts (numnp %d, nsd %d, nshg %d)", I.numnp, I.nsd, I.nshg);
    g->x.resize((size_t)I.numnp * I.nsd);
    rc = phgpu_io_readdatablock(o.fd, "co-ordinates", g->x.data(), I.numnp * I.nsd, "double", "binary");
    if (rc) return rc;
    // genblkPosix: one "connectivity interior?" block per topology, in file order
    for (int b = 0; b < I.nelblk; ++b) {
        int h[7] = {0, 0, 0, 0, 0, 0, 0};
        rc = read_int_header(o.fd, "connectivity interior?", h, 7);
        if (rc) return rc;
        phgpu_topblock t{h[0], h[1], h[2], h[3], 0, 0, h[6], 0};
        if (t.neltp < 0 || t.nshl <= 0) return fail(PHGPU_ERR_INVALID, "geombc_open: bad interior block %d", b);
        std::vector<int> e((size_t)t.neltp * t.nshl);
        rc = phgpu_io_readdatablock(o.fd, "connectivity interior?", e.data(), (int)e.size(), "integer", "binary");
        if (rc) return rc;
        g->interior.push_back(t);
        g->ien.push_back(std::move(e));
    }
    // the headers of the nodal arrays give their sizes (readnblk.f:303-372 read them into nshg, numpbc)
    rc = read_int_header(o.fd, "bc mapping array", &I.nshg, 1);
    if (rc) return rc;
    if (I.nshg <= 0 || I.numpbc < 0) return fail(PHGPU_ERR_INVALID, "geombc_open: bad bc mapping array size");
    g->nBC.resize(I.nshg);
    rc = phgpu_io_readdatablock(o.fd, "bc mapping array", g->nBC.data(), I.nshg, "integer", "binary");
    if (rc) return rc;
    rc = read_int_header(o.fd, "bc codes array", &I.numpbc, 1);
    if (rc) return rc;
    g->iBCtmp.resize(I.numpbc);
    rc = phgpu_io_readdatablock(o.fd, "bc codes array", g->iBCtmp.data(), I.numpbc, "integer", "binary");
    if (rc) return rc;
    int bsize = 0;
    rc = phgpu_io_readheader(o.fd, "boundary condition array", &bsize, 1, "double", "binary");
    if (rc) return rc;
    I.nbccols = I.numpbc > 0 ? bsize / I.numpbc : 0;
    if (I.numpbc > 0 && I.nbccols < ndof + 7)
        return fail(PHGPU_ERR_INVALID, "geombc_open: boundary condition array has %d columns, needs %d", I.nbccols, ndof + 7);
    g->BCinp.resize(std::max(bsize, 0));
    rc = phgpu_io_readdatablock(o.fd, "boundary condition array", g->BCinp.data(), bsize, "double", "binary");
    if (rc) return rc;
    rc = read_int_header(o.fd, "periodic masters array", &I.nshg, 1);
    if (rc) return rc;
    if (I.nshg != (int)g->nBC.size()) return fail(PHGPU_ERR_INVALID, "geombc_open: periodic masters array of %d nodes, bc mapping array of %zu", I.nshg, g->nBC.size());
    g->iper.resize(I.nshg);
    rc = phgpu_io_readdatablock(o.fd, "periodic masters array", g->iper.data(), I.nshg, "integer", "binary");
    if (rc) return rc;
    // genbkbPosix: "connectivity boundary?", "nbc codes?", "nbc values?" per block
    const int ndBCB = ndof + 1;
    for (int b = 0; b < I.nelblb; ++b) {
        int h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        rc = read_int_header(o.fd, "connectivity boundary?", h, 8);
        if (rc) return rc;
        phgpu_topblock t{h[0], h[1], h[2], h[3], h[4], h[5], h[6], h[7]};
        if (t.neltp < 0 || t.nshl <= 0 || t.nshlb < t.nenbl || t.nenbl < 0)
            return fail(PHGPU_ERR_INVALID, "geombc_open: bad boundary block %d", b);
        const size_t ne = t.neltp;
        std::vector<int> e(ne * t.nshl), codes(ne * 2);
        std::vector<double> vals(ne * ndBCB, 0.0);
        rc = phgpu_io_readdatablock(o.fd, "connectivity boundary?", e.data(), (int)e.size(), "integer", "binary");
        int hh[8];
        if (!rc) rc = read_int_header(o.fd, "nbc codes?", hh, 8);
        if (!rc) rc = phgpu_io_readdatablock(o.fd, "nbc codes?", codes.data(), (int)codes.size(), "integer", "binary");
        if (!rc) rc = read_int_header(o.fd, "nbc values?", hh, 8);
        if (!rc) rc = phgpu_io_readdatablock(o.fd, "nbc values?", vals.data(), (int)vals.size(), "double", "binary");
        if (rc) return rc;
        // zero what the flux codes do not set (genbkbPosix.f:126-142)
        for (size_t i = 0; i < ne; ++i) {
            int c = codes[i];
            auto v = [&](int col) -> double& { return vals[(size_t)(col - 1) * ne + i]; };
            if (!(c & 1)) v(1) = 0.0;
            if (!(c & 2)) v(2) = 0.0;
            if (!(c & 8)) v(6) = 0.0;
            for (int k = 6; k <= ndof && ndBCB > 6; ++k)
                if (!((c >> (k - 1)) & 1)) v(k + 1) = 0.0;
            if (!(c & 4)) v(3) = v(4) = v(5) = 0.0;
        }
        // gensvb: the element values on the first nenbl face nodes, zero on the others
        std::vector<double> bcb(ne * t.nshlb * ndBCB, 0.0);
        for (int j = 0; j < ndBCB; ++j)
            for (int a = 0; a < t.nenbl; ++a)
                for (size_t i = 0; i < ne; ++i)
                    bcb[((size_t)j * t.nshlb + a) * ne + i] = vals[(size_t)j * ne + i];
        g->boundary.push_back(t);
        g->ienb.push_back(std::move(e));
        g->iBCB.push_back(std::move(codes));
        g->BCB.push_back(std::move(bcb));
    }
    *out = g.release();
    return PHGPU_OK;
}

int phgpu_io_geombc_free(phgpu_geombc* g) {
    delete g;
    return PHGPU_OK;
}

int phgpu_io_geombc_info(const phgpu_geombc* g, phgpu_geombc_info* info) {
    if (!g || !info) return fail(PHGPU_ERR_INVALID, "geombc_info: null argument");
    *info = g->info;
    return PHGPU_OK;
}

int phgpu_io_geombc_arrays(const phgpu_geombc* g, double* x, int* nBC, int* iBCtmp, double* BCinp, int* iper) {
    if (!g) return fail(PHGPU_ERR_INVALID, "geombc_arrays: null handle");
    if (x) std::copy(g->x.begin(), g->x.end(), x);
    if (nBC) std::copy(g->nBC.begin(), g->nBC.end(), nBC);
    if (iBCtmp) std::copy(g->iBCtmp.begin(), g->iBCtmp.end(), iBCtmp);
    if (BCinp) std::copy(g->BCinp.begin(), g->BCinp.end(), BCinp);
    if (iper) std::copy(g->iper.begin(), g->iper.end(), iper);
    return PHGPU_OK;
}

int phgpu_io_geombc_interior(const phgpu_geombc* g, int iblk, phgpu_topblock* blk, int* ien) {
    if (!g || iblk < 0 || iblk >= (int)g->interior.size()) return fail(PHGPU_ERR_INVALID, "geombc_interior: bad block");
    if (blk) *blk = g->interior[iblk];
    if (ien) std::copy(g->ien[iblk].begin(), g->ien[iblk].end(), ien);
    return PHGPU_OK;
}

int phgpu_io_geombc_boundary(const phgpu_geombc* g, int iblk, phgpu_topblock* blk, int* ienb, int* iBCB,
                             double* BCB) {
    if (!g || iblk < 0 || iblk >= (int)g->boundary.size()) return fail(PHGPU_ERR_INVALID, "geombc_boundary: bad block");
    if (blk) *blk = g->boundary[iblk];
    if (ienb) std::copy(g->ienb[iblk].begin(), g->ienb[iblk].end(), ienb);
    if (iBCB) std::copy(g->iBCB[iblk].begin(), g->iBCB[iblk].end(), iBCB);
    if (BCB) std::copy(g->BCB[iblk].begin(), g->BCB[iblk].end(), BCB);
    return PHGPU_OK;
}

int phgpu_io_genibc(int nshg, int numpbc, const int* nBC, const int* iBCtmp, int* iBC) {
    if (nshg <= 0 || numpbc < 0 || !nBC || !iBC || (numpbc > 0 && !iBCtmp))
        return fail(PHGPU_ERR_INVALID, "genibc: bad argument");
    for (int n = 0; n < nshg; ++n) {
        int m = nBC[n];
        if (numpbc == 0 || m == 0) {
            iBC[n] = 0;
            continue;
        }
        if (m < 1 || m > numpbc) return fail(PHGPU_ERR_INVALID, "genibc: nBC(%d) = %d out of range", n + 1, m);
        iBC[n] = iBCtmp[m - 1];
    }
    return PHGPU_OK;
}

int phgpu_io_genbc(int nshg, int numpbc, int ndof, const int* nBC, const double* BCinp, int ldbc, const int* iBC,
                   double* BC) {
    if (nshg <= 0 || numpbc < 0 || ndof < 5 || !nBC || !iBC || !BC || (numpbc > 0 && (!BCinp || ldbc < ndof + 7)))
        return fail(PHGPU_ERR_INVALID, "genbc: bad argument");
    const size_t N = nshg;
    const int nt = ndof + 7, nbc = ndof + 1, nsclr = ndof - 5;
    // BCtmp(nshg, ndof+7): D T P c11 c12 c13 M1 c21 c22 c23 M2 theta S1 ... (genbc.f:38-57)
    std::vector<double> t(N * nt, 0.0);
    auto T = [&](size_t n, int c) -> double& { return t[(size_t)(c - 1) * N + n]; };
    for (size_t n = 0; n < N; ++n) {
        int m = nBC[n];
        if (numpbc == 0 || m == 0) continue;
        if (m < 1 || m > numpbc) return fail(PHGPU_ERR_INVALID, "genbc: nBC(%zu) = %d out of range", n + 1, m);
        for (int c = 1; c <= nt; ++c) T(n, c) = BCinp[(size_t)(c - 1) * numpbc + (m - 1)];
    }
    for (size_t n = 0; n < N; ++n)
        if (T(n, 12) != 0.0) return fail(PHGPU_ERR_UNSUPPORTED, "genbc: periodic rotation (BCinp(:,12)) is not supported");
    std::fill(BC, BC + N * nbc, 0.0);
    auto B = [&](size_t n, int c) -> double& { return BC[(size_t)(c - 1) * N + n]; };
    for (size_t n = 0; n < N; ++n) {
        const int ib = iBC[n];
        for (int s = 1; s <= nsclr; ++s)
            if ((ib >> (5 + s)) & 1) B(n, 6 + s) = T(n, 12 + s);
        if (ib & 1) B(n, 1) = T(n, 1);  // density
        if (ib & 2) B(n, 2) = T(n, 2);  // temperature
        if (ib & 4) B(n, 1) = T(n, 3);  // pressure (same slot as density)
        const int v = (ib >> 3) & 7;
        // one constrained velocity component: the constraint c.u = M scaled by the pivot (genbc1.f:42-60, 107-114)
        auto single = [&](int piv, int o1, int o2) {
            double s = T(n, 4) * T(n, 4) + T(n, 5) * T(n, 5) + T(n, 6) * T(n, 6);
            B(n, 3) = s * T(n, 7) / T(n, piv);
            B(n, 4) = T(n, o1) / T(n, piv);
            B(n, 5) = T(n, o2) / T(n, piv);
        };
        // two constrained components (genbc1.f:62-105, 116-171, 173-220): normalise both
        // constraint vectors, eliminate, and keep the reduced pair of equations
        auto two = [&](int zero1, int zero2) {
            if (T(n, zero1) == 0.0 || T(n, zero2) == 0.0)
                for (int c = 0; c < 4; ++c) std::swap(T(n, 4 + c), T(n, 8 + c));
            double a = std::sqrt(T(n, 4) * T(n, 4) + T(n, 5) * T(n, 5) + T(n, 6) * T(n, 6));
            T(n, 4) /= a;
            T(n, 5) /= a;
            T(n, 6) /= a;
            T(n, 7) *= a;
            double b = std::sqrt(T(n, 8) * T(n, 8) + T(n, 9) * T(n, 9) + T(n, 10) * T(n, 10));
            T(n, 8) /= b;
            T(n, 9) /= b;
            T(n, 10) /= b;
            T(n, 11) *= b;
        };
        switch (v) {
            case 1: single(4, 5, 6); break;
            case 2: single(5, 4, 6); break;
            case 4: single(6, 4, 5); break;
            case 3: {  // x1 & x2
                two(4, 9);
                T(n, 4) = T(n, 9) * T(n, 4) - T(n, 5) * T(n, 8);
                T(n, 6) = T(n, 9) * T(n, 6) - T(n, 5) * T(n, 10);
                T(n, 7) = T(n, 9) * T(n, 7) - T(n, 5) * T(n, 11);
                B(n, 3) = T(n, 7) / T(n, 4);
                B(n, 4) = T(n, 6) / T(n, 4);
                T(n, 9) = T(n, 4) * T(n, 9);
                T(n, 10) = T(n, 4) * T(n, 10) - T(n, 8) * T(n, 6);
                T(n, 11) = T(n, 4) * T(n, 11) - T(n, 8) * T(n, 7);
                B(n, 5) = T(n, 11) / T(n, 9);
                B(n, 6) = T(n, 10) / T(n, 9);
                break;
            }
            case 5: {  // x1 & x3
                two(4, 10);
                T(n, 4) = T(n, 10) * T(n, 4) - T(n, 6) * T(n, 8);
                T(n, 5) = T(n, 10) * T(n, 5) - T(n, 6) * T(n, 9);
                T(n, 7) = T(n, 10) * T(n, 7) - T(n, 6) * T(n, 11);
                B(n, 3) = T(n, 7) / T(n, 4);
                B(n, 4) = T(n, 5) / T(n, 4);
                T(n, 9) = T(n, 4) * T(n, 9) - T(n, 8) * T(n, 5);
                T(n, 10) = T(n, 4) * T(n, 10);
                T(n, 11) = T(n, 4) * T(n, 11) - T(n, 8) * T(n, 7);
                B(n, 5) = T(n, 11) / T(n, 10);
                B(n, 6) = T(n, 9) / T(n, 10);
                break;
            }
            case 6: {  // x2 & x3
                two(5, 10);
                T(n, 4) = T(n, 10) * T(n, 4) - T(n, 6) * T(n, 8);
                T(n, 5) = T(n, 10) * T(n, 5) - T(n, 6) * T(n, 9);
                T(n, 7) = T(n, 10) * T(n, 7) - T(n, 6) * T(n, 11);
                B(n, 3) = T(n, 7) / T(n, 5);
                B(n, 4) = T(n, 4) / T(n, 5);
                T(n, 8) = T(n, 5) * T(n, 8) - T(n, 9) * T(n, 4);
                T(n, 10) = T(n, 5) * T(n, 10);
                T(n, 11) = T(n, 5) * T(n, 11) - T(n, 9) * T(n, 7);
                B(n, 5) = T(n, 11) / T(n, 10);
                B(n, 6) = T(n, 8) / T(n, 10);
                break;
            }
            case 7:  // all three: magnitude times direction
                B(n, 3) = T(n, 7) * T(n, 4);
                B(n, 4) = T(n, 7) * T(n, 5);
                B(n, 5) = T(n, 7) * T(n, 6);
                break;
            default: break;
        }
    }
    return PHGPU_OK;
}

// ---- checkphasta ------------------------------------------------------------------------

static std::set<int> restart_steps(const char* dir) {
    std::set<int> steps;
    DIR* d = opendir(dir);
    if (!d) return steps;
    while (dirent* e = readdir(d)) {
        int ts, part;
        if (std::sscanf(e->d_name, "restart.%d.%d", &ts, &part) == 2) steps.insert(ts);
    }
    closedir(d);
    return steps;
}

static int read_solution(const char* dir, int step, int rank, std::vector<double>& sol) {
    std::string name = part_name(dir, "restart." + std::to_string(step) + ".", rank);
    Open o(name, "read");
    if (!o.fd) return fail(PHGPU_ERR_IO, "checkphasta: unable to open %s", name.c_str());
    int h[3] = {0, 0, 0};
    int rc = phgpu_io_readheader(o.fd, "solution", h, 3, "integer", "binary");
    if (rc) return rc;
    sol.assign((size_t)h[0] * h[1], 0.0);
    return phgpu_io_readdatablock(o.fd, "solution", sol.data(), (int)sol.size(), "double", "binary");
}

int phgpu_io_checkphasta(const char* left, const char* right, int nparts, double* maxdiff, int* nsteps) {
    if (!left || !right || nparts < 1 || !maxdiff) return fail(PHGPU_ERR_INVALID, "checkphasta: bad argument");
    DIR* dl = opendir(left);
    DIR* dr = opendir(right);
    if (dl) closedir(dl);
    if (dr) closedir(dr);
    if (!dl || !dr) return fail(PHGPU_ERR_IO, "checkphasta: cannot open case directory");
    std::set<int> l = restart_steps(left), r = restart_steps(right), common;
    std::set_intersection(l.begin(), l.end(), r.begin(), r.end(), std::inserter(common, common.begin()));
    double m = 0.0;
    std::vector<double> a, b;
    for (int step : common)
        for (int p = 0; p < nparts; ++p) {
            int rc = read_solution(left, step, p, a);
            if (!rc) rc = read_solution(right, step, p, b);
            if (rc) return rc;
            if (a.size() != b.size())
                return fail(PHGPU_ERR_INVALID, "checkphasta: solution sizes differ: %zu, %zu", a.size(), b.size());
            for (size_t i = 0; i < a.size(); ++i) m = std::max(m, std::fabs(a[i] - b[i]));
        }
    *maxdiff = m;
    if (nsteps) *nsteps = (int)common.size();
    return PHGPU_OK;
}

}  // extern "C"

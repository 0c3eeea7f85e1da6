// nova-gb300: loaders for nova's raw (comma-separated) POMDP and MDP files.
//
// Replaces the reference's Python readers FileLoader.load_raw_pomdp and
// load_raw_mdp (python/nova/file_loader.py:74-209), which parse every value
// with Python loops; the layout is the same:
//
//   POMDP: header  n, ns, m, z, r, rz, k, s0, horizon, gamma
//          S rows (a, s) -> ns successors;  T rows (a, s) -> ns probabilities
//          O rows (a, o) -> n values over s';  R rows (i, a) -> n values over s
//          Z rows i -> rz states;  B rows i -> rz values
//   MDP:   header  n, ns, m, k, s0, ng, horizon, gamma;  goals row (ng values)
//          S rows, T rows, R rows as above
//
// Values are read as the reference reads them (Python int()/float(), i.e.
// strtol/strtod) and stored as the POMDP/MDP structs' int/float; of the k
// reward functions, rewardIndex selects one (the reference's default
// scalarisation takes the first).

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nova/error_codes.h>
#include <nova/mdp/mdp.h>
#include <nova/mdp/utilities/mdp_model_cpu.h>
#include <nova/nova_gb300.h>
#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/utilities/pomdp_model_cpu.h>

using nova::MDP;
using nova::POMDP;

namespace {

#define LOAD_ERR(fn, msg) fprintf(stderr, "Error[%s]: %s\n", fn, msg)

// The file as rows of comma-separated fields (empty trailing lines dropped).
bool read_rows(const char *path, std::vector<std::vector<std::string>> &rows) {
    FILE *f = fopen(path, "r");
    if (f == nullptr) return false;
    std::string line;
    int c;
    auto flush = [&]() {
        std::vector<std::string> fields;
        size_t start = 0;
        for (size_t i = 0; i <= line.size(); i++) {
            if (i == line.size() || line[i] == ',') {
                fields.push_back(line.substr(start, i - start));
                start = i + 1;
            }
        }
        if (!(fields.size() == 1 && fields[0].empty())) rows.push_back(fields);
        line.clear();
    };
    while ((c = fgetc(f)) != EOF) {
        if (c == '\n') flush();
        else if (c != '\r') line.push_back((char)c);
    }
    if (!line.empty()) flush();
    fclose(f);
    return true;
}

bool to_long(const std::string &s, long &out) {
    const char *p = s.c_str();
    while (*p == ' ' || *p == '\t') p++;
    char *end = nullptr;
    errno = 0;
    out = strtol(p, &end, 10);
    if (end == p || errno != 0) return false;
    while (*end == ' ' || *end == '\t') end++;
    return *end == '\0';
}

bool to_double(const std::string &s, double &out) {
    const char *p = s.c_str();
    while (*p == ' ' || *p == '\t') p++;
    char *end = nullptr;
    errno = 0;
    out = strtod(p, &end);
    if (end == p) return false;
    while (*end == ' ' || *end == '\t') end++;
    return *end == '\0';
}

struct Reader {
    const std::vector<std::vector<std::string>> &rows;
    bool ok = true;
    long i(size_t r, size_t c) {
        long v = 0;
        if (r >= rows.size() || c >= rows[r].size() || !to_long(rows[r][c], v)) ok = false;
        return v;
    }
    double d(size_t r, size_t c) {
        double v = 0.0;
        if (r >= rows.size() || c >= rows[r].size() || !to_double(rows[r][c], v)) ok = false;
        return v;
    }
};

}  // namespace

extern "C" int nova_load_raw_pomdp(const char *path, POMDP *pomdp, unsigned int rewardIndex) {
    static const char *fn = "nova_load_raw_pomdp";
    if (path == nullptr || pomdp == nullptr || pomdp->S != nullptr) {
        LOAD_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    std::vector<std::vector<std::string>> rows;
    if (!read_rows(path, rows) || rows.empty()) {
        LOAD_ERR(fn, "Failed to read the file.");
        return NOVA_ERROR_INVALID_DATA;
    }
    Reader rd{rows};
    const long n = rd.i(0, 0), ns = rd.i(0, 1), m = rd.i(0, 2), z = rd.i(0, 3), r = rd.i(0, 4), rz = rd.i(0, 5);
    const long k = rd.i(0, 6);
    const long horizon = rd.i(0, 8);
    const double gamma = rd.d(0, 9);
    if (!rd.ok || n <= 0 || ns <= 0 || m <= 0 || z <= 0 || r <= 0 || rz <= 0 || k <= 0 || horizon <= 0 ||
            (long)rewardIndex >= k) {
        LOAD_ERR(fn, "Invalid header.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = nova::pomdp_initialize_cpu(pomdp, (unsigned)n, (unsigned)ns, (unsigned)m, (unsigned)z, (unsigned)r,
                                        (unsigned)rz, (float)gamma, (unsigned)horizon);
    if (rc != NOVA_SUCCESS) return rc;
    size_t off = 1;
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++)
            for (long l = 0; l < ns; l++)
                pomdp->S[(s * m + a) * ns + l] = (int)rd.i(off + n * a + s, l);
    off += (size_t)(n * m);
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++)
            for (long l = 0; l < ns; l++)
                pomdp->T[(s * m + a) * ns + l] = (float)rd.d(off + n * a + s, l);
    off += (size_t)(n * m);
    for (long a = 0; a < m; a++)
        for (long sp = 0; sp < n; sp++)
            for (long o = 0; o < z; o++)
                pomdp->O[(a * n + sp) * z + o] = (float)rd.d(off + z * a + o, sp);
    off += (size_t)(m * z);
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++)
            pomdp->R[s * m + a] = (float)rd.d(off + m * (long)rewardIndex + a, s);
    off += (size_t)(k * m);
    for (long i = 0; i < r; i++)
        for (long j = 0; j < rz; j++) pomdp->Z[i * rz + j] = (int)rd.i(off + i, j);
    off += (size_t)r;
    for (long i = 0; i < r; i++)
        for (long j = 0; j < rz; j++) pomdp->B[i * rz + j] = (float)rd.d(off + i, j);
    if (!rd.ok) {
        nova::pomdp_uninitialize_cpu(pomdp);
        LOAD_ERR(fn, "Missing or malformed values.");
        return NOVA_ERROR_INVALID_DATA;
    }
    return NOVA_SUCCESS;
}

extern "C" int nova_load_raw_mdp(const char *path, MDP *mdp, unsigned int rewardIndex) {
    static const char *fn = "nova_load_raw_mdp";
    if (path == nullptr || mdp == nullptr || mdp->S != nullptr) {
        LOAD_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    std::vector<std::vector<std::string>> rows;
    if (!read_rows(path, rows) || rows.empty()) {
        LOAD_ERR(fn, "Failed to read the file.");
        return NOVA_ERROR_INVALID_DATA;
    }
    Reader rd{rows};
    const long n = rd.i(0, 0), ns = rd.i(0, 1), m = rd.i(0, 2), k = rd.i(0, 3), s0 = rd.i(0, 4), ng = rd.i(0, 5);
    const long horizon = rd.i(0, 6);
    const double gamma = rd.d(0, 7);
    if (!rd.ok || n <= 0 || ns <= 0 || m <= 0 || k <= 0 || ng < 0 || horizon <= 0 || (long)rewardIndex >= k) {
        LOAD_ERR(fn, "Invalid header.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = nova::mdp_initialize_cpu(mdp, (unsigned)n, (unsigned)ns, (unsigned)m, (float)gamma, (unsigned)horizon,
                                      0.0f, (unsigned)s0, (unsigned)ng);
    if (rc != NOVA_SUCCESS) return rc;
    for (long g = 0; g < ng; g++) mdp->goals[g] = (unsigned)rd.i(1, g);
    size_t off = 2;
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++)
            for (long l = 0; l < ns; l++) mdp->S[(s * m + a) * ns + l] = (int)rd.i(off + n * a + s, l);
    off += (size_t)(n * m);
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++)
            for (long l = 0; l < ns; l++) mdp->T[(s * m + a) * ns + l] = (float)rd.d(off + n * a + s, l);
    off += (size_t)(n * m);
    // epsilon = (Rmax - Rmin) / 1000 over the selected reward, as the reference
    // computes it (unused by the raw format's fixed horizon).
    double rmax = -1e300, rmin = 1e300;
    for (long s = 0; s < n; s++)
        for (long a = 0; a < m; a++) {
            const double v = rd.d(off + m * (long)rewardIndex + a, s);
            mdp->R[s * m + a] = (float)v;
            if (v > rmax) rmax = v;
            if (v < rmin) rmin = v;
        }
    mdp->epsilon = (float)((rmax - rmin) / 1000.0);
    if (!rd.ok) {
        nova::mdp_uninitialize_cpu(mdp);
        LOAD_ERR(fn, "Missing or malformed values.");
        return NOVA_ERROR_INVALID_DATA;
    }
    return NOVA_SUCCESS;
}

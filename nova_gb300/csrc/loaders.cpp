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

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
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

// ---------------------------------------------------------------------------
// Cassandra-format POMDP files, read with the rules of the reference's
// FileLoader.load_cassandra (python/nova/file_loader.py:211-588):
//
//   * Lines lose everything from '#' on and their outer white space; empty
//     lines are dropped. A line containing ':' starts a new statement; the
//     lines that follow it, up to the next such line, belong to it
//     (:222-268). Lines before the first statement are ignored.
//   * A statement "name: p1 : p2 : ... : last" (:270-343) with no parameter
//     stores the next line's tokens (one line) or the list of the following
//     lines' tokens; with one parameter on a line of its own it stores that
//     parameter's tokens; with several parameters on one line it stores, under
//     the key (p1, ..., first token of last), the second token of last; with
//     following lines it stores those lines' tokens (one line) or token lists
//     under the key (p1, ..., last). Keys keep their first position when
//     redefined and take the new value (Python dictionaries).
//   * The model is then built (:345-588): states/actions/observations as a
//     count or a list of names; start as a distribution over all states or a
//     single state's name, then "start include" / "start exclude" lists, each
//     giving one belief; T as matrix/row/entry statements, "uniform" and
//     "identity", with '*' wildcards, each positive value appended to the
//     successor list of (s, a) in statement order (ns is the longest list,
//     shorter lists padded with -1 and 0); O likewise into a dense
//     [m][n][z] array (later statements overwrite); R(s, a) = the mean of the
//     statement's numbers (numpy's pairwise summation), later statements
//     overwriting, and the horizon int(log(eps / (Rmax - Rmin)) / log(gamma))
//     + 1 with eps = (Rmax - Rmin) / 1000. The discount defaults to 0.9.
//
// Two differences from running the reference's code, both where it fails:
// the reference's start test compares the token list with "uniform" (never
// equal), so "start: uniform" is looked up as a state name and fails there
// too; and its reward statements call numpy's removed np.float alias, read
// here as Python's float.
// ---------------------------------------------------------------------------

namespace {

struct CVal {  // a parsed value: a string, a token list, or a list of token lists
    enum Kind { Str, List, Mat } kind = List;
    std::string s;
    std::vector<std::string> list;
    std::vector<std::vector<std::string>> mat;
};

struct CVar {
    bool isDict = false;
    CVal plain;
    std::vector<std::pair<std::vector<std::string>, CVal>> dict;  // insertion order
    std::map<std::vector<std::string>, size_t> where;             // key -> position in dict
    void put(const std::vector<std::string> &key, CVal &&v) {
        auto it = where.find(key);
        if (it != where.end()) {
            dict[it->second].second = std::move(v);
            return;
        }
        where.emplace(key, dict.size());
        dict.emplace_back(key, std::move(v));
    }
};

struct CassandraError {};

bool py_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

std::string py_strip(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && py_space(s[a])) a++;
    while (b > a && py_space(s[b - 1])) b--;
    return s.substr(a, b - a);
}

std::vector<std::string> py_split_ws(const std::string &s) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && py_space(s[i])) i++;
        size_t j = i;
        while (j < s.size() && !py_space(s[j])) j++;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

std::vector<std::string> py_split_colon(const std::string &s) {
    std::vector<std::string> out;
    size_t start = 0;
    for (size_t i = 0; i <= s.size(); i++)
        if (i == s.size() || s[i] == ':') {
            out.push_back(s.substr(start, i - start));
            start = i + 1;
        }
    return out;
}

double py_float(const std::string &tok) {
    double v;
    if (!to_double(tok, v)) throw CassandraError();
    return v;
}

long py_int(const std::string &tok) {
    long v;
    if (!to_long(tok, v)) throw CassandraError();
    return v;
}

// Python's v[i][j] on a parsed value, as a string (indexing a string gives
// its i-th character).
std::string elem2(const CVal &v, size_t i, size_t j) {
    if (v.kind == CVal::Mat) {
        if (i >= v.mat.size() || j >= v.mat[i].size()) throw CassandraError();
        return v.mat[i][j];
    }
    if (v.kind == CVal::List) {
        if (i >= v.list.size() || j >= v.list[i].size()) throw CassandraError();
        return std::string(1, v.list[i][j]);
    }
    if (i >= v.s.size() || j != 0) throw CassandraError();
    return std::string(1, v.s[i]);
}

// Python's float(v[i]): a token (or a character of a string); a list fails.
double elem1f(const CVal &v, size_t i) {
    if (v.kind == CVal::Mat) throw CassandraError();
    if (v.kind == CVal::List) {
        if (i >= v.list.size()) throw CassandraError();
        return py_float(v.list[i]);
    }
    if (i >= v.s.size()) throw CassandraError();
    return py_float(std::string(1, v.s[i]));
}

bool first_is(const CVal &v, const char *word) {
    if (v.kind == CVal::List) {
        if (v.list.empty()) throw CassandraError();
        return v.list[0] == word;
    }
    if (v.kind == CVal::Mat) {
        if (v.mat.empty()) throw CassandraError();
        return false;
    }
    if (v.s.empty()) throw CassandraError();
    return false;
}

double scalar_f(const CVal &v) {
    if (v.kind != CVal::Str) throw CassandraError();
    return py_float(v.s);
}

// numpy's float64 sum: pairwise, blocks of up to 128 added through eight
// running sums, sequentially below 8 terms.
double pairwise_sum(const double *a, size_t n) {
    if (n < 8) {
        double r = 0.0;
        for (size_t i = 0; i < n; i++) r += a[i];
        return r;
    }
    if (n <= 128) {
        double r[8];
        for (int j = 0; j < 8; j++) r[j] = a[j];
        size_t i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; j++) r[j] += a[i + j];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; i++) res += a[i];
        return res;
    }
    size_t n2 = n / 2;
    n2 -= n2 % 8;
    return pairwise_sum(a, n2) + pairwise_sum(a + n2, n - n2);
}

// mean of np.array([value]).astype(float)
double value_mean(const CVal &v) {
    std::vector<double> xs;
    if (v.kind == CVal::Str) {
        xs.push_back(py_float(v.s));
    } else if (v.kind == CVal::List) {
        for (auto &t : v.list) xs.push_back(py_float(t));
    } else {
        for (auto &row : v.mat) {
            if (row.size() != v.mat[0].size()) throw CassandraError();  // ragged: not an array
            for (auto &t : row) xs.push_back(py_float(t));
        }
    }
    return pairwise_sum(xs.data(), xs.size()) / (double)xs.size();
}

// Names of states, actions or observations: a count or a list of names.
std::vector<std::string> names_of(std::map<std::string, CVar> &vars, const char *what) {
    auto it = vars.find(what);
    if (it == vars.end() || it->second.isDict) throw CassandraError();
    const CVal &v = it->second.plain;
    std::vector<std::string> toks;
    if (v.kind == CVal::List) toks = v.list;
    else if (v.kind == CVal::Mat) throw CassandraError();
    else throw CassandraError();
    if (toks.size() == 1) {
        const long count = py_int(toks[0]);
        if (count < 0) throw CassandraError();
        std::vector<std::string> out;
        for (long i = 0; i < count; i++) out.push_back(std::to_string(i));
        return out;
    }
    return toks;
}

size_t index_of(const std::vector<std::string> &names, const std::string &x) {
    for (size_t i = 0; i < names.size(); i++)
        if (names[i] == x) return i;
    throw CassandraError();
}

std::vector<size_t> selection(const std::vector<std::string> &names, const std::string &x) {
    std::vector<size_t> out;
    if (x == "*") {
        for (size_t i = 0; i < names.size(); i++) out.push_back(i);
    } else {
        out.push_back(index_of(names, x));
    }
    return out;
}

std::map<std::string, CVar> parse_cassandra(const char *path) {
    FILE *f = fopen(path, "r");
    if (f == nullptr) throw CassandraError();
    std::vector<std::vector<std::string>> data(1);
    std::string line;
    int c;
    auto flush = [&]() {
        std::string l = line;
        line.clear();
        const size_t hash = l.find('#');
        if (hash != std::string::npos) l = l.substr(0, hash);
        l = py_strip(l);
        if (l.empty()) return;
        if (l.find(':') != std::string::npos) data.emplace_back();
        data.back().push_back(l);
    };
    // Universal newlines: "\n", "\r\n" and "\r" end a line.
    while ((c = fgetc(f)) != EOF) {
        if (c == '\n') {
            flush();
        } else if (c == '\r') {
            flush();
            const int c2 = fgetc(f);
            if (c2 != '\n' && c2 != EOF) ungetc(c2, f);
        } else {
            line.push_back((char)c);
        }
    }
    flush();
    fclose(f);
    std::map<std::string, CVar> vars;
    vars["values"].plain.kind = CVal::Str;  // the reference's dictionary starts as {'values': "reward"}
    vars["values"].plain.s = "reward";
    for (size_t di = 1; di < data.size(); di++) {
        const auto &d = data[di];
        const std::vector<std::string> parts = py_split_colon(d[0]);
        const std::string variable = py_strip(parts[0]);
        std::vector<std::string> params;
        for (size_t k = 1; k < parts.size(); k++)
            if (!parts[k].empty()) params.push_back(py_strip(parts[k]));
        const bool exists = vars.count(variable) != 0;
        CVar &var = vars[variable];
        auto lines_value = [&]() {
            CVal v;
            if (d.size() == 2) {
                v.kind = CVal::List;
                v.list = py_split_ws(d[1]);
            } else {
                v.kind = CVal::Mat;
                for (size_t k = 1; k < d.size(); k++) v.mat.push_back(py_split_ws(d[k]));
            }
            return v;
        };
        if (params.empty()) {
            var.isDict = false;
            var.dict.clear();
            var.where.clear();
            var.plain = lines_value();
            continue;
        }
        const std::vector<std::string> tokenOrList = py_split_ws(params.back());
        if (d.size() == 1 && params.size() == 1) {
            var.isDict = false;
            var.dict.clear();
            var.where.clear();
            var.plain = CVal();
            var.plain.kind = CVal::List;
            var.plain.list = tokenOrList;
            continue;
        }
        // Keyed statements need a dictionary: storing into a list fails.
        if (exists && !var.isDict) throw CassandraError();
        var.isDict = true;
        std::vector<std::string> key(params.begin(), params.end() - 1);
        if (d.size() == 1) {
            if (tokenOrList.size() < 2) throw CassandraError();
            key.push_back(tokenOrList[0]);
            CVal v;
            v.kind = CVal::Str;
            v.s = tokenOrList[1];
            var.put(key, std::move(v));
        } else {
            key.push_back(params.back());
            var.put(key, lines_value());
        }
    }
    return vars;
}

}  // namespace

extern "C" int nova_load_cassandra_pomdp(const char *path, POMDP *pomdp, double *Rmin, double *Rmax) {
    static const char *fn = "nova_load_cassandra_pomdp";
    if (path == nullptr || pomdp == nullptr || pomdp->S != nullptr) {
        LOAD_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    try {
        std::map<std::string, CVar> vars = parse_cassandra(path);
        double gamma = 0.9;
        {
            auto it = vars.find("discount");
            if (it != vars.end() && !it->second.isDict) {
                const CVal &v = it->second.plain;
                if (v.kind == CVal::List) {
                    if (v.list.empty()) throw CassandraError();
                    gamma = py_float(v.list[0]);
                } else {
                    throw CassandraError();
                }
            }
        }
        const std::vector<std::string> states = names_of(vars, "states");
        const std::vector<std::string> actions = names_of(vars, "actions");
        const std::vector<std::string> observations = names_of(vars, "observations");
        const size_t n = states.size(), m = actions.size(), z = observations.size();
        // Initial belief: r = 1.
        bool haveStart = false;
        std::vector<int> Zb;
        std::vector<double> Bb;
        // A keyed start statement makes the reference's lookups raise KeyError,
        // which it skips.
        if (vars.count("start") && !vars["start"].isDict) {
            const CVar &sv = vars["start"];
            if (sv.plain.kind != CVal::List) throw CassandraError();
            const auto &st = sv.plain.list;
            if (st.size() == 1) {
                Zb = {(int)index_of(states, st[0])};
                Bb = {1.0};
            } else {
                if (st.size() < n) throw CassandraError();
                for (size_t s = 0; s < n; s++) {
                    Zb.push_back((int)s);
                    Bb.push_back(py_float(st[s]));
                }
            }
            haveStart = true;
        }
        if (vars.count("start include") && !vars["start include"].isDict) {
            const CVar &sv = vars["start include"];
            if (sv.plain.kind != CVal::List) throw CassandraError();
            const auto &inc = sv.plain.list;
            Zb.clear();
            Bb.clear();
            for (auto &x : inc) {
                Zb.push_back((int)index_of(states, x));
                Bb.push_back(1.0 / (double)inc.size());
            }
            haveStart = true;
        }
        if (vars.count("start exclude") && !vars["start exclude"].isDict) {
            const CVar &sv = vars["start exclude"];
            if (sv.plain.kind != CVal::List) throw CassandraError();
            const auto &exc = sv.plain.list;
            if (exc.size() > n) throw CassandraError();
            const size_t rz = n - exc.size();
            std::vector<int> keep;
            for (size_t s = 0; s < n; s++)
                if (std::find(exc.begin(), exc.end(), states[s]) == exc.end()) keep.push_back((int)s);
            if (keep.size() < rz) throw CassandraError();
            keep.resize(rz);
            Zb = keep;
            Bb.assign(rz, 1.0 / (double)rz);
            haveStart = true;
        }
        if (!haveStart || Zb.empty()) throw CassandraError();
        // Transitions.
        if (!vars.count("T") || !vars["T"].isDict) throw CassandraError();
        std::vector<std::vector<int>> Sl(n * m);
        std::vector<std::vector<double>> Tl(n * m);
        auto add = [&](size_t s, size_t a, size_t sp, double p) {
            if (p > 0.0) {
                Sl[s * m + a].push_back((int)sp);
                Tl[s * m + a].push_back(p);
            }
        };
        for (auto &kv : vars["T"].dict) {
            const auto &key = kv.first;
            const CVal &value = kv.second;
            const std::vector<size_t> as = selection(actions, key[0]);
            if (key.size() == 1) {
                const bool uniform = first_is(value, "uniform");
                const bool identity = !uniform && first_is(value, "identity");
                for (size_t a : as)
                    for (size_t s = 0; s < n; s++)
                        for (size_t sp = 0; sp < n; sp++)
                            add(s, a, sp, uniform ? 1.0 / (double)n
                                                  : identity ? (s == sp ? 1.0 : 0.0) : py_float(elem2(value, s, sp)));
            } else if (key.size() == 2) {
                const bool uniform = first_is(value, "uniform");
                const std::vector<size_t> ss = selection(states, key[1]);
                for (size_t a : as)
                    for (size_t s : ss)
                        for (size_t sp = 0; sp < n; sp++) add(s, a, sp, uniform ? 1.0 / (double)n : elem1f(value, sp));
            } else if (key.size() == 3) {
                const std::vector<size_t> ss = selection(states, key[1]);
                const std::vector<size_t> sps = selection(states, key[2]);
                const double p = scalar_f(value);
                for (size_t a : as)
                    for (size_t s : ss)
                        for (size_t sp : sps) add(s, a, sp, p);
            }
        }
        size_t ns = 1;
        for (auto &l : Sl) ns = std::max(ns, l.size());
        // Observations.
        std::vector<double> Od(m * n * z, 0.0);
        if (vars.count("O")) {
            if (!vars["O"].isDict) throw CassandraError();
            for (auto &kv : vars["O"].dict) {
                const auto &key = kv.first;
                const CVal &value = kv.second;
                const std::vector<size_t> as = selection(actions, key[0]);
                if (key.size() == 1) {
                    const bool uniform = first_is(value, "uniform");
                    for (size_t a : as)
                        for (size_t sp = 0; sp < n; sp++)
                            for (size_t o = 0; o < z; o++)
                                Od[(a * n + sp) * z + o] =
                                    uniform ? 1.0 / (double)z : py_float(elem2(value, sp, o));
                } else if (key.size() == 2) {
                    const bool uniform = first_is(value, "uniform");
                    const std::vector<size_t> sps = selection(states, key[1]);
                    for (size_t a : as)
                        for (size_t sp : sps)
                            for (size_t o = 0; o < z; o++)
                                Od[(a * n + sp) * z + o] = uniform ? 1.0 / (double)z : elem1f(value, o);
                } else if (key.size() == 3) {
                    const std::vector<size_t> sps = selection(states, key[1]);
                    const std::vector<size_t> os = selection(observations, key[2]);
                    const double p = scalar_f(value);
                    for (size_t a : as)
                        for (size_t sp : sps)
                            for (size_t o : os) Od[(a * n + sp) * z + o] = p;
                }
            }
        }
        // Rewards and horizon.
        if (!vars.count("R") || !vars["R"].isDict) throw CassandraError();
        std::vector<double> Rd(n * m, 0.0);
        for (auto &kv : vars["R"].dict) {
            const auto &key = kv.first;
            if (key.size() < 2) throw CassandraError();
            const std::vector<size_t> as = selection(actions, key[0]);
            const std::vector<size_t> ss = selection(states, key[1]);
            const double mean = value_mean(kv.second);
            for (size_t a : as)
                for (size_t s : ss) Rd[s * m + a] = mean;
        }
        if (n * m == 0) throw CassandraError();
        double rmax = Rd[0], rmin = Rd[0];
        bool nan = false;
        for (double v : Rd) {
            if (v != v) nan = true;
            rmax = std::max(rmax, v);
            rmin = std::min(rmin, v);
        }
        if (nan) throw CassandraError();
        const double eps = (rmax - rmin) / 1000.0;
        const double hx = std::log(eps / (rmax - rmin)) / std::log(gamma);
        if (!(hx == hx) || std::fabs(hx) > 2e9) throw CassandraError();
        const long horizon = (long)hx + 1;  // int() truncates toward zero
        if (horizon <= 0 || n == 0 || z == 0) throw CassandraError();
        const size_t rz = Zb.size();
        int rc = nova::pomdp_initialize_cpu(pomdp, (unsigned)n, (unsigned)ns, (unsigned)m, (unsigned)z, 1u,
                                            (unsigned)rz, (float)gamma, (unsigned)horizon);
        if (rc != NOVA_SUCCESS) return rc;
        for (size_t s = 0; s < n; s++)
            for (size_t a = 0; a < m; a++)
                for (size_t l = 0; l < ns; l++) {
                    const auto &sl = Sl[s * m + a];
                    const size_t idx = (s * m + a) * ns + l;
                    pomdp->S[idx] = l < sl.size() ? sl[l] : -1;
                    pomdp->T[idx] = l < sl.size() ? (float)Tl[s * m + a][l] : 0.0f;
                }
        for (size_t i = 0; i < m * n * z; i++) pomdp->O[i] = (float)Od[i];
        for (size_t i = 0; i < n * m; i++) pomdp->R[i] = (float)Rd[i];
        for (size_t k = 0; k < rz; k++) {
            pomdp->Z[k] = Zb[k];
            pomdp->B[k] = (float)Bb[k];
        }
        if (Rmin != nullptr) *Rmin = rmin;
        if (Rmax != nullptr) *Rmax = rmax;
        return NOVA_SUCCESS;
    } catch (const CassandraError &) {
        LOAD_ERR(fn, "Failed to read the file as a Cassandra-format POMDP.");
        return NOVA_ERROR_INVALID_DATA;
    }
}

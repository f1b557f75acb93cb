// Native host-side input helpers (include/phylocsf_host.h): ECM reader, Newick
// parser with CamlPaml node numbering, candidate-region enumeration and leaf
// packing.  Reference behaviour (paths relative to mlin/PhyloCSF):
//   ECM.import_parameters   src/ECM.ml:18-72
//   Newick lexer / parser   lib/CamlPaml/NewickLexer.mll:1-14, NewickParser.mly:1-25
//   T.of_newick             lib/CamlPaml/T.ml:57-112
//   find_orfs, candidate_regions   src/PhyloCSF.ml:134-217
//   pleaves, Codon64.index/is      src/PhyloCSF.ml:219-246, lib/CamlPaml/Code.ml:18-30,138-141
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <thread>
#include <string>
#include <vector>

#include "../../include/phylocsf_host.h"

void pcsf_internal_set_error(const std::string &msg);

namespace {

int fail(int code, const std::string &msg)
{
    pcsf_internal_set_error(msg);
    return code;
}

// Code.DNA.index over ACGT/acgt; -1 otherwise
inline int dna_index(char c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return -1;
    }
}

// split on single spaces, trim, drop empties (Str.split re_sp + String.trim)
std::vector<std::string> fields(const std::string &line)
{
    std::vector<std::string> out;
    size_t i = 0;
    while (i <= line.size()) {
        size_t j = line.find(' ', i);
        if (j == std::string::npos) j = line.size();
        std::string s = line.substr(i, j - i);
        size_t a = 0, b = s.size();
        while (a < b && std::isspace((unsigned char)s[a])) a++;
        while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
        if (b > a) out.push_back(s.substr(a, b - a));
        i = j + 1;
    }
    return out;
}

bool parse_double(const std::string &s, double &v)
{
    char *end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0' && !s.empty();
}

// ---- Newick -----------------------------------------------------------------

struct NNode {
    std::vector<std::unique_ptr<NNode>> kids;
    std::string label;
    bool has_bl = false;
    double bl = 0.0;
};

struct NewickParser {
    enum Kind { LP, RP, COMMA, COLON, LEN, LABEL, END };
    struct Tok {
        Kind k;
        std::string s;
        double v;
    };
    std::vector<Tok> toks;
    size_t pos = 0;
    std::string err;

    static bool labchar(char c) { return std::isalnum((unsigned char)c) || c == '_' || c == '.'; }

    bool lex(const char *t)
    {
        size_t n = std::strlen(t), i = 0;
        while (i < n) {
            char c = t[i];
            if (c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == ';') { i++; continue; }
            if (c == '(') { toks.push_back({LP, "", 0}); i++; continue; }
            if (c == ')') { toks.push_back({RP, "", 0}); i++; continue; }
            if (c == ',') { toks.push_back({COMMA, "", 0}); i++; continue; }
            if (c == ':') { toks.push_back({COLON, "", 0}); i++; continue; }
            if (labchar(c)) {
                // longest match; a tie goes to the branch-length rule ([0-9.]+), listed first
                size_t j = i, k = i;
                while (j < n && labchar(t[j])) j++;
                while (k < n && (std::isdigit((unsigned char)t[k]) || t[k] == '.')) k++;
                if (k >= j) {
                    std::string s(t + i, k - i);
                    double v;
                    if (!parse_double(s, v)) { err = "Newick: bad branch length " + s; return false; }
                    toks.push_back({LEN, s, v});
                    i = k;
                } else {
                    toks.push_back({LABEL, std::string(t + i, j - i), 0});
                    i = j;
                }
                continue;
            }
            err = std::string("Newick: unexpected character '") + c + "'";
            return false;
        }
        toks.push_back({END, "", 0});
        return true;
    }
    Kind peek() const { return toks[pos].k; }
    bool take(Kind k, Tok *out = nullptr)
    {
        if (toks[pos].k != k) { err = "Newick: syntax error"; return false; }
        if (out) *out = toks[pos];
        pos++;
        return true;
    }
    bool label(NNode &nd)
    {
        Tok t;
        if (peek() == LABEL) {
            take(LABEL, &t);
            nd.label = t.s;
            if (peek() == COLON) {
                take(COLON);
                if (!take(LEN, &t)) return false;
                nd.has_bl = true;
                nd.bl = t.v;
            }
            return true;
        }
        if (!take(COLON)) return false;
        if (!take(LEN, &t)) return false;
        nd.has_bl = true;
        nd.bl = t.v;
        return true;
    }
    std::unique_ptr<NNode> node()
    {
        auto nd = std::make_unique<NNode>();
        if (peek() == LP) {
            take(LP);
            for (;;) {
                auto k = node();
                if (!k) return nullptr;
                nd->kids.push_back(std::move(k));
                if (peek() == COMMA) { take(COMMA); continue; }
                break;
            }
            if (!take(RP)) return nullptr;
            if (peek() == LABEL || peek() == COLON)
                if (!label(*nd)) return nullptr;
            return nd;
        }
        if (!label(*nd)) return nullptr;
        return nd;
    }
};

}  // namespace

extern "C" {

int pcsf_read_ecm(const char *path, double *S, double *pi)
{
    if (!path || !S || !pi) return fail(PCSF_EINVAL, "pcsf_read_ecm: null argument");
    std::ifstream f(path);
    if (!f) return fail(PCSF_EINVAL, std::string("pcsf_read_ecm: cannot open ") + path);
    std::vector<std::string> lines;
    std::string line;
    while (std::getline(f, line)) lines.push_back(line);
    if (lines.size() < 71) return fail(PCSF_EINVAL, "ECM.import_parameters: file too short");
    std::vector<std::vector<double>> raw(63);
    for (int i = 0; i < 63; i++) {
        for (auto &s : fields(lines[i])) {
            double v;
            if (!parse_double(s, v)) return fail(PCSF_EINVAL, "ECM.import_parameters: bad number " + s);
            raw[i].push_back(v);
        }
        if ((int)raw[i].size() < i + 1) return fail(PCSF_EINVAL, "ECM.import_parameters: short row");
    }
    for (int i = 0; i < 64; i++)
        for (int j = 0; j < 64; j++)
            S[i * 64 + j] = (i > j) ? raw[i - 1][j] : (i < j) ? raw[j - 1][i] : 0.0;
    if (!fields(lines[63]).empty()) return fail(PCSF_EINVAL, "ECM.import_parameters");
    auto pf = fields(lines[64]);
    if (pf.size() != 64) return fail(PCSF_EINVAL, "ECM.import_parameters: expected 64 frequencies");
    for (int i = 0; i < 64; i++)
        if (!parse_double(pf[i], pi[i])) return fail(PCSF_EINVAL, "ECM.import_parameters: bad frequency " + pf[i]);
    std::vector<std::string> codons;
    for (int li = 67; li <= 70; li++)
        for (auto &s : fields(lines[li])) codons.push_back(s);
    if (codons.size() != 64) return fail(PCSF_EINVAL, "ECM.import_parameters: incorrect codon order");
    for (int i = 0; i < 64; i++) {
        const std::string &c = codons[i];
        if (c.size() != 3) return fail(PCSF_EINVAL, "ECM.import_parameters: codon " + c);
        int a = dna_index(c[0]), b = dna_index(c[1]), d = dna_index(c[2]);
        if (a < 0 || b < 0 || d < 0 || 16 * a + 4 * b + d != i)
            return fail(PCSF_EINVAL, "ECM.import_parameters: incorrect codon order");
    }
    return PCSF_OK;
}

int pcsf_parse_newick(const char *text, int32_t max_nodes, int32_t *n_leaves, int32_t *parent, double *branch,
                      char *labels, int32_t label_stride)
{
    if (!text || !n_leaves || !parent || !branch) return fail(PCSF_EINVAL, "pcsf_parse_newick: null argument");
    NewickParser p;
    if (!p.lex(text)) return fail(PCSF_EINVAL, p.err);
    auto root = p.node();
    if (!root) return fail(PCSF_EINVAL, p.err.empty() ? "Newick: syntax error" : p.err);
    if (p.peek() != NewickParser::END) return fail(PCSF_EINVAL, "Newick: trailing tokens");
    // T.of_newick: leaves left to right, internal nodes post-order
    std::vector<const NNode *> leaves;
    std::vector<const NNode *> st{root.get()};
    bool bif = true;
    std::function<void(const NNode *)> find = [&](const NNode *x) {
        if (x->kids.empty()) { leaves.push_back(x); return; }
        if (x->kids.size() != 2) { bif = false; return; }
        find(x->kids[0].get());
        find(x->kids[1].get());
    };
    find(root.get());
    if (!bif) return fail(PCSF_EINVAL, "CamlPaml.T.of_newick: input is not a rooted, bifurcating tree");
    int nl = (int)leaves.size();
    int n = 2 * nl - 1;
    if (nl < 2) return fail(PCSF_EINVAL, "CamlPaml.T.of_newick: input is not a rooted, bifurcating tree");
    if (n > max_nodes) return fail(PCSF_ERANGE, "pcsf_parse_newick: tree has more nodes than max_nodes");
    int next = nl - 1, leaf_i = 0;
    bool label_ok = true;
    std::function<int(const NNode *)> fill = [&](const NNode *x) -> int {
        int i;
        if (x->kids.empty()) {
            i = leaf_i++;
        } else {
            int lc = fill(x->kids[0].get());
            int rc = fill(x->kids[1].get());
            i = ++next;
            parent[lc] = i;
            parent[rc] = i;
        }
        branch[i] = x->has_bl ? x->bl : NAN;
        if (labels && label_stride > 0) {
            if ((int)x->label.size() >= label_stride) label_ok = false;
            else std::memcpy(labels + (size_t)i * label_stride, x->label.c_str(), x->label.size() + 1);
        }
        return i;
    };
    int r = fill(root.get());
    parent[r] = -1;
    if (!label_ok) return fail(PCSF_ERANGE, "pcsf_parse_newick: a label is longer than label_stride-1");
    *n_leaves = nl;
    return PCSF_OK;
}

}  // extern "C"

namespace {

inline char up(char c) { return (char)std::toupper((unsigned char)c); }
inline bool codon_is(const char *p, const char *a)
{
    return up(p[0]) == a[0] && up(p[1]) == a[1] && up(p[2]) == a[2];
}
inline bool is_stop(const char *p) { return codon_is(p, "TAA") || codon_is(p, "TAG") || codon_is(p, "TGA"); }

typedef std::pair<int64_t, int64_t> Orf;

// find_orfs (PhyloCSF.ml:134-196).  The reference builds its lists by
// prepending; `orfs` here is kept in that most-recent-first order.
std::vector<Orf> find_orfs(const char *dna, int64_t n, int64_t ofs, int mode, int min_codons)
{
    const bool atg = mode == PCSF_ORF_ATGSTOP;
    std::vector<Orf> orfs;      // most recent first
    std::vector<int64_t> starts;   // most recent first
    for (int64_t lo = ofs; lo <= n - 3; lo++) {
        if ((lo - ofs) % 3 != 0) continue;
        int64_t hi = lo + 2;
        if ((!atg && starts.empty() && !is_stop(dna + lo)) || (atg && codon_is(dna + lo, "ATG")))
            starts.insert(starts.begin(), lo);
        if (hi + 3 < n && is_stop(dna + hi + 1)) {
            for (int64_t s : starts)
                if (hi > s + 2) orfs.insert(orfs.begin(), Orf(s, hi));
            starts.clear();
        }
    }
    if (!atg)
        for (int64_t s : starts) {
            int64_t rem = n - s;
            orfs.insert(orfs.begin(), Orf(s, s + (rem / 3) * 3 - 1));
        }
    if (mode == PCSF_ORF_STOPSTOP3) {
        std::vector<Orf> all;
        for (auto &o : orfs) {
            std::vector<Orf> sub{o};
            int64_t lo = o.first, hi = o.second, cod = (hi - lo + 1) / 3;
            int64_t lo2 = lo + (cod / 3) * 3;
            if (lo2 > lo) sub.insert(sub.begin(), Orf(lo2, hi));
            int64_t lo3 = lo + (2 * cod / 3) * 3;
            if (lo3 > lo2 && lo3 > lo) sub.insert(sub.begin(), Orf(lo3, hi));
            all.insert(all.end(), sub.begin(), sub.end());
        }
        orfs = all;
    }
    if (mode == PCSF_ORF_TOFIRSTSTOP && !orfs.empty()) {
        Orf first = orfs.back();
        orfs.clear();
        if (first.first == ofs) orfs.push_back(first);
    }
    if (mode == PCSF_ORF_FROMLASTSTOP && !orfs.empty()) {
        Orf last = orfs.front();
        orfs.clear();
        if (n - last.second <= 3) orfs.push_back(last);
    }
    if (mode == PCSF_ORF_TOORFROMSTOP && !orfs.empty()) {
        Orf first = orfs.back(), last = orfs.front();
        orfs.clear();
        if (first.first == ofs) orfs.push_back(first);
        if (n - last.second <= 3 && first != last) orfs.insert(orfs.begin(), last);
    }
    std::vector<Orf> out;
    for (auto it = orfs.rbegin(); it != orfs.rend(); ++it)
        if ((it->second - it->first + 1) / 3 >= min_codons) out.push_back(*it);
    return out;
}

bool revcomp(const char *s, int64_t n, std::string &out)
{
    out.assign((size_t)n, ' ');
    for (int64_t i = 0; i < n; i++) {
        char c = s[i], r;
        switch (c) {
        case 'A': r = 'T'; break;
        case 'G': r = 'C'; break;
        case 'C': r = 'G'; break;
        case 'T': r = 'A'; break;
        case 'a': r = 't'; break;
        case 'g': r = 'c'; break;
        case 'c': r = 'g'; break;
        case 't': r = 'a'; break;
        case 'N': r = 'N'; break;
        case 'n': r = 'n'; break;
        case '-': r = '-'; break;
        default: return false;
        }
        out[(size_t)(n - 1 - i)] = r;
    }
    return true;
}

}  // namespace

extern "C" {

int pcsf_candidate_regions(const char *ref, int64_t len, int32_t frames, int32_t orf_mode, int32_t min_codons,
                           int32_t cap, int32_t *rc, int64_t *lo, int64_t *hi, int32_t *count)
{
    if (!ref || !count || len < 0) return fail(PCSF_EINVAL, "pcsf_candidate_regions: bad argument");
    if (frames != 1 && frames != 3 && frames != 6) return fail(PCSF_EINVAL, "invalid reading frame");
    if (orf_mode < PCSF_ORF_ASIS || orf_mode > PCSF_ORF_TOORFROMSTOP) return fail(PCSF_EINVAL, "invalid ORF search mode");
    struct R { int32_t rc; int64_t lo, hi; };
    std::vector<R> out;
    if (orf_mode == PCSF_ORF_ASIS) {
        int64_t h = len - 1;
        out.push_back({0, 0, h});
        if (frames != 1) { out.push_back({0, 1, h}); out.push_back({0, 2, h}); }
        if (frames == 6) { out.push_back({1, 0, h}); out.push_back({1, 1, h}); out.push_back({1, 2, h}); }
    } else {
        int nf = frames == 1 ? 1 : 3;
        for (int o = 0; o < nf; o++)
            for (auto &x : find_orfs(ref, len, o, orf_mode, min_codons)) out.push_back({0, x.first, x.second});
        if (frames == 6) {
            std::string r;
            if (!revcomp(ref, len, r)) return fail(PCSF_EINVAL, "unrecognized nucleotide");
            for (int o = 0; o < 3; o++)
                for (auto &x : find_orfs(r.data(), len, o, orf_mode, min_codons)) out.push_back({1, x.first, x.second});
        }
    }
    *count = (int32_t)out.size();
    for (int i = 0; i < (int)out.size() && i < cap; i++) {
        if (rc) rc[i] = out[i].rc;
        if (lo) lo[i] = out[i].lo;
        if (hi) hi[i] = out[i].hi;
    }
    return PCSF_OK;
}

int pcsf_bls_columns(int32_t n_leaves, const int32_t *parent, const double *branch, const int32_t *leaf_rows,
                     int32_t n_rows, const char *const *rows, int64_t len, double *out)
{
    if (n_leaves < 2 || !parent || !branch || !leaf_rows || (n_rows > 0 && !rows) || len < 0 || (len > 0 && !out))
        return fail(PCSF_EINVAL, "pcsf_bls_columns: bad argument");
    const int nl = n_leaves, n = 2 * nl - 1;
    for (int i = 0; i < n - 1; i++)
        if (parent[i] <= i || parent[i] >= n) return fail(PCSF_EINVAL, "pcsf_bls_columns: tree is not in T order");
    for (int l = 0; l < nl; l++)
        if (leaf_rows[l] >= n_rows) return fail(PCSF_EINVAL, "pcsf_bls_columns: leaf row out of range");
    std::vector<int> below(n);
    for (int64_t c = 0; c < len; c++) {
        std::fill(below.begin(), below.end(), 0);
        for (int l = 0; l < nl; l++) {
            const int r = leaf_rows[l];
            if (r < 0) continue;
            const char x = rows[r][c];
            below[l] = (x == '-' || x == '.' || x == 'N') ? 0 : 1;
        }
        for (int i = 0; i < n - 1; i++) below[parent[i]] += below[i];   // children precede parents
        const int total = below[n - 1];
        double t = 0.0;
        for (int i = 0; i < n - 1; i++)
            if (below[i] > 0 && below[i] < total) t += branch[i];
        out[c] = t;
    }
    return PCSF_OK;
}

int pcsf_pack_regions(int32_t n_leaves, const int32_t *leaf_rows, int32_t n_rows, const char *const *rows_fwd,
                      const char *const *rows_rc, int64_t len, int32_t n_regions, const int32_t *rc,
                      const int64_t *lo, const int64_t *hi, int64_t *col_offsets, uint8_t *leaves)
{
    if (n_leaves < 1 || !leaf_rows || !rows_fwd || n_regions < 0 || !col_offsets || (n_regions > 0 && (!lo || !hi)))
        return fail(PCSF_EINVAL, "pcsf_pack_regions: bad argument");
    for (int l = 0; l < n_leaves; l++)
        if (leaf_rows[l] >= n_rows) return fail(PCSF_EINVAL, "pcsf_pack_regions: leaf row out of range");
    int64_t total = 0;
    col_offsets[0] = 0;
    for (int r = 0; r < n_regions; r++) {
        int64_t a = lo[r], b = hi[r];
        if (a < 0 || b >= len) return fail(PCSF_EINVAL, "pcsf_pack_regions: region out of range");
        const bool use_rc = rc && rc[r];
        if (use_rc && !rows_rc) return fail(PCSF_EINVAL, "pcsf_pack_regions: reverse-complemented rows missing");
        const char *const *rows = use_rc ? rows_rc : rows_fwd;
        for (int64_t pos = a; pos + 2 <= b; pos += 3) {
            if (leaves) {
                uint8_t *col = leaves + (size_t)total * n_leaves;
                for (int l = 0; l < n_leaves; l++) {
                    int row = leaf_rows[l];
                    uint8_t code = PCSF_MARGINALIZE;
                    if (row >= 0) {
                        const char *p = rows[row] + pos;
                        int x = dna_index(p[0]), y = dna_index(p[1]), z = dna_index(p[2]);
                        if (x >= 0 && y >= 0 && z >= 0) code = (uint8_t)(16 * x + 4 * y + z);
                    }
                    col[l] = code;
                }
            }
            total++;
        }
        col_offsets[r + 1] = total;
    }
    return PCSF_OK;
}

}  // extern "C"

namespace {

inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct ColumnRng {
    uint64_t s;
    ColumnRng(uint64_t seed, uint64_t col) : s(mix64(seed * 0x9E3779B97F4A7C15ULL + col + 1)) {}
    double next()
    {
        s += 0x9E3779B97F4A7C15ULL;
        return (double)(mix64(s) >> 11) * (1.0 / 9007199254740992.0);
    }
};

// smallest j with u < cum[j] (cum ascending, cum[63] ~ 1)
inline int draw(const double *cum, double u)
{
    int lo = 0, hi = 63;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (u < cum[mid]) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

}  // namespace

extern "C" int pcsf_simulate(int32_t n_leaves, const int32_t *parent, int32_t n_models, const double *P,
                             const double *prior, int32_t n_regions, const int64_t *col_offsets,
                             const int32_t *region_model, const double *gap_frac, int32_t reject_stop_leaf0,
                             uint64_t seed, int32_t n_threads, uint8_t *leaves)
{
    if (n_leaves < 2 || !parent || n_models < 1 || !P || !prior || n_regions < 0 || !col_offsets || !region_model ||
        !leaves)
        return fail(PCSF_EINVAL, "pcsf_simulate: bad argument");
    const int nl = n_leaves, n = 2 * nl - 1, nbr = n - 1;
    for (int i = 0; i < n - 1; i++)
        if (parent[i] <= i || parent[i] >= n) return fail(PCSF_EINVAL, "pcsf_simulate: tree is not in T order");
    for (int r = 0; r < n_regions; r++)
        if (region_model[r] < 0 || region_model[r] >= n_models) return fail(PCSF_EINVAL, "pcsf_simulate: bad model");
    // cumulative rows and prior
    std::vector<double> cum((size_t)n_models * nbr * 64 * 64), cpr((size_t)n_models * 64);
    for (int m = 0; m < n_models; m++) {
        double c = 0;
        for (int a = 0; a < 64; a++) cpr[m * 64 + a] = (c += prior[m * 64 + a]);
        for (int b = 0; b < nbr; b++)
            for (int a = 0; a < 64; a++) {
                const double *row = P + (((size_t)m * nbr + b) * 64 + a) * 64;
                double *cr = cum.data() + (((size_t)m * nbr + b) * 64 + a) * 64;
                double t = 0;
                for (int j = 0; j < 64; j++) cr[j] = (t += row[j]);
            }
    }
    const int64_t total = col_offsets[n_regions];
    int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<int64_t>(nt, std::max<int64_t>(1, total / 4096));
    auto work = [&](int tid) {
        std::vector<int> st(n);
        int r = 0;
        int64_t c0 = total * tid / nt, c1 = total * (tid + 1) / nt;
        while (r < n_regions && col_offsets[r + 1] <= c0) r++;
        for (int64_t c = c0; c < c1; c++) {
            while (r < n_regions && col_offsets[r + 1] <= c) r++;
            const int m = region_model[r];
            ColumnRng rng(seed, (uint64_t)c);
            for (int attempt = 0; attempt < 1000; attempt++) {
                st[n - 1] = draw(cpr.data() + m * 64, rng.next() * cpr[m * 64 + 63]);
                for (int i = n - 2; i >= 0; i--) {
                    const double *cr = cum.data() + (((size_t)m * nbr + i) * 64 + st[parent[i]]) * 64;
                    st[i] = draw(cr, rng.next() * cr[63]);
                }
                const int s0 = st[0];
                if (!(reject_stop_leaf0 && (s0 == 48 || s0 == 50 || s0 == 56))) break;   // TAA TAG TGA
            }
            uint8_t *col = leaves + (size_t)c * nl;
            for (int l = 0; l < nl; l++) {
                uint8_t code = (uint8_t)st[l];
                if (gap_frac && rng.next() < gap_frac[(size_t)r * nl + l]) code = PCSF_MARGINALIZE;
                col[l] = code;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    return PCSF_OK;
}

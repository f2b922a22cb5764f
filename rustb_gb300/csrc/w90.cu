// Wannier90 tight-binding tables (seedname_hr.dat, _r.dat, _wsvec.dat) read
// natively into the hop-table layout the device model takes (ham (nR, N, N)
// complex, R = 0 first, hamR (nR, 3)), following Wannier90::from_hr
// (src/wannier90.rs:49-1203):
//   _hr.dat   header, nsta (line 2), n_R (line 3), degeneracy weights until the
//             first line holding a '.', then n_R blocks of nsta^2 lines
//             "a b c i j re im"; line ind_i * nsta + ind_j of block r gives
//             ham[R][ind_j][ind_i] = (re + i im) / weight[r] (the file is
//             column-major); R from the block's first line; R = 0 goes to
//             index 0, the others are appended in file order; zero_energy is
//             subtracted from the R = 0 diagonal (:85-245).
//   _r.dat    n_R blocks of nsta^2 lines "a b c i j xr xi yr yi zr zi" from line
//             4, each R matched to the Hamiltonian's, divided by the HR weight
//             of the same block (:771-880).
//   _wsvec.dat  Wigner-Seitz refolding: each (R, i, j) entry is spread over its
//             listed shifts R + T with weight 1/n (:882-1142).
//   r-matrix Hermitisation over all R rows but the last (:1146-1167).
// Only the positions of values are used, as the reference does (the i, j
// columns are not read).  The data lines of _hr.dat are parsed by all host
// threads: newlines are counted per byte chunk, then each thread converts the
// lines that start in its chunk (std::from_chars, correctly rounded as Rust's
// f64 parser).  Host code only: the tables are uploaded by tbg_model_create.

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "tbgpu_internal.cuh"

struct tbg_w90 {
    int64_t nsta = 0;
    std::vector<int64_t> hamR;       // (nR, 3), R = 0 first
    std::vector<double> ham;         // (nR, nsta, nsta) complex
    std::vector<int64_t> weights;    // per _hr.dat block
    bool has_r = false;
    std::vector<double> rmat;        // (nR, 3, nsta, nsta) complex
    int64_t nR() const { return (int64_t)hamR.size() / 3; }
};

namespace tbg {
namespace {

int file_error(const std::string& file, const std::string& msg) {
    return set_error(TBG_E_FILE_PARSE, "Failed to parse data from file '" + file + "': " + msg);
}

bool read_file(const char* path, std::string& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? std::fread(&out[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    out.resize(got);
    return true;
}

// Line [b, e) of the buffer (BufRead::lines: '\n' split, one trailing '\r' dropped).
struct Line {
    const char* b;
    const char* e;
};

Line line_at(const std::string& s, size_t& pos) {
    const char* base = s.data();
    const size_t n = s.size();
    const size_t start = pos;
    const void* nl = std::memchr(base + start, '\n', n - start);
    size_t end = nl ? (size_t)((const char*)nl - base) : n;
    pos = nl ? end + 1 : n;
    if (end > start && base[end - 1] == '\r') --end;
    return {base + start, base + end};
}

// Next whitespace-separated token of [p, e); false at the end of the line.
bool next_token(const char*& p, const char* e, const char*& tb, const char*& te) {
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\v' || *p == '\f' || *p == '\r')) ++p;
    if (p >= e) return false;
    tb = p;
    while (p < e && !(*p == ' ' || *p == '\t' || *p == '\v' || *p == '\f' || *p == '\r')) ++p;
    te = p;
    return true;
}

bool parse_f64(const char* b, const char* e, double& v) {
    if (b < e && *b == '+') ++b;  // Rust's f64 parser takes a leading '+'
    const auto r = std::from_chars(b, e, v);
    return r.ec == std::errc() && r.ptr == e;
}

bool parse_i64(const char* b, const char* e, int64_t& v) {
    if (b < e && *b == '+') ++b;
    const auto r = std::from_chars(b, e, v);
    return r.ec == std::errc() && r.ptr == e;
}

bool parse_u64(const char* b, const char* e, int64_t& v) {
    if (b < e && *b == '+') ++b;
    if (b < e && *b == '-') return false;
    uint64_t u = 0;
    const auto r = std::from_chars(b, e, u);
    if (r.ec != std::errc() || r.ptr != e || u > (uint64_t)INT64_MAX) return false;
    v = (int64_t)u;
    return true;
}

std::string trimmed(Line l) {
    while (l.b < l.e && std::isspace((unsigned char)*l.b)) ++l.b;
    while (l.e > l.b && std::isspace((unsigned char)l.e[-1])) --l.e;
    return std::string(l.b, l.e);
}

int64_t find_R(const std::vector<int64_t>& hamR, int64_t a, int64_t b, int64_t c) {
    const int64_t n = (int64_t)hamR.size() / 3;
    for (int64_t r = 0; r < n; ++r)
        if (hamR[3 * r] == a && hamR[3 * r + 1] == b && hamR[3 * r + 2] == c) return r;
    return -1;
}

unsigned n_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return std::max(1u, std::min(h ? h : 1u, 64u));
}

// Data lines [first, first + count) of a buffer whose line `first` starts at
// byte `off`: calls fn(line_index - first, Line) on all host threads.
template <class Fn>
int parallel_lines(const std::string& s, size_t off, int64_t count, Fn fn) {
    if (count <= 0) return 0;
    const unsigned T = n_threads();
    const size_t n = s.size();
    const size_t span = n - off;
    std::vector<size_t> cut(T + 1);
    for (unsigned t = 0; t <= T; ++t) cut[t] = off + span * t / T;
    // move every cut to the start of a line
    for (unsigned t = 1; t < T; ++t) {
        const void* nl = std::memchr(s.data() + cut[t] - 1, '\n', n - (cut[t] - 1));
        cut[t] = nl ? (size_t)((const char*)nl - s.data()) + 1 : n;
        cut[t] = std::max(cut[t], cut[t - 1]);
    }
    std::vector<int64_t> lines_before(T + 1, 0);
    {
        std::vector<std::thread> th;
        std::vector<int64_t> cnt(T, 0);
        for (unsigned t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                int64_t c = 0;
                for (size_t p = cut[t]; p < cut[t + 1];) {
                    const void* nl = std::memchr(s.data() + p, '\n', cut[t + 1] - p);
                    if (!nl) {
                        ++c;  // last line without a newline
                        break;
                    }
                    ++c;
                    p = (size_t)((const char*)nl - s.data()) + 1;
                }
                cnt[t] = c;
            });
        for (auto& x : th) x.join();
        for (unsigned t = 0; t < T; ++t) lines_before[t + 1] = lines_before[t] + cnt[t];
    }
    if (lines_before[T] < count) return -1;  // file too short
    std::vector<int> err(T, 0);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            int64_t L = lines_before[t];
            size_t p = cut[t];
            while (p < cut[t + 1] && L < count) {
                const Line l = line_at(s, p);
                const int e = fn(L, l);
                if (e) {
                    err[t] = e;
                    return;
                }
                ++L;
            }
        });
    for (auto& x : th) x.join();
    for (unsigned t = 0; t < T; ++t)
        if (err[t]) return err[t];
    return 0;
}

}  // namespace
}  // namespace tbg

using namespace tbg;

extern "C" {

int tbg_w90_read_hr(const char* hr_path, double zero_energy, tbg_w90** out) {
    if (!hr_path || !out) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    const std::string file(hr_path);
    std::string s;
    if (!read_file(hr_path, s))
        return set_error(TBG_E_FILE_OPEN, "Failed to create file '" + file + "': Unable to open HR file");
    size_t pos = 0;
    std::vector<Line> head;
    // header (comment), nsta, n_R
    for (int i = 0; i < 3 && pos < s.size(); ++i) head.push_back(line_at(s, pos));
    if (head.size() < 3) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _hr.dat has fewer than 3 lines");
    int64_t nsta = 0, nR = 0;
    {
        const std::string t = trimmed(head[1]);
        if (!parse_u64(t.data(), t.data() + t.size(), nsta))
            return file_error(file, "Failed to parse nsta: invalid digit found in string");
        const std::string u = trimmed(head[2]);
        if (!parse_u64(u.data(), u.data() + u.size(), nR))
            return file_error(file, "Failed to parse n_R: invalid digit found in string");
    }
    if (nsta == 0) return set_error(TBG_E_INVALID_MODEL, "model has no orbitals");
    if (nsta > 4096) return set_error(TBG_E_UNSUPPORTED, "nsta > 4096 is not supported");
    // weights until the first line holding a '.'
    std::vector<int64_t> weights;
    size_t data_off = s.size();
    bool found = false;
    while (pos < s.size()) {
        const size_t here = pos;
        const Line l = line_at(s, pos);
        if (std::memchr(l.b, '.', (size_t)(l.e - l.b))) {
            data_off = here;
            found = true;
            break;
        }
        const char* p = l.b;
        const char *tb, *te;
        while (next_token(p, l.e, tb, te)) {
            int64_t w = 0;
            if (!parse_u64(tb, te, w)) return file_error(file, "Failed to parse weight: invalid digit found in string");
            weights.push_back(w);
        }
    }
    if (!found && nR > 0)
        return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: no Hamiltonian lines in _hr.dat");
    if ((int64_t)weights.size() < nR)
        return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: fewer degeneracy weights than R vectors");
    const int64_t NN = nsta * nsta;
    // parse all blocks in file order into (nR, nsta, nsta), R per block
    std::vector<double> raw((size_t)(nR * NN) * 2, 0.0);
    std::vector<int64_t> Rv((size_t)nR * 3, 0);
    std::vector<std::string> msgs(1);
    const int rc = parallel_lines(s, data_off, nR * NN, [&](int64_t L, Line l) -> int {
        const int64_t blk = L / NN, e = L % NN, ind_i = e / nsta, ind_j = e % nsta;
        const char* p = l.b;
        const char *tb, *te;
        double v[2];
        int tok = 0;
        int64_t rv[3];
        while (tok < 7 && next_token(p, l.e, tb, te)) {
            if (e == 0 && tok < 3) {
                if (!parse_i64(tb, te, rv[tok])) return 3;  // R component
            }
            if (tok >= 5) {
                if (!parse_f64(tb, te, v[tok - 5])) return tok == 5 ? 5 : 6;
            }
            ++tok;
        }
        if (e == 0 && tok < 3) return 2;
        if (tok < 6) return 7;
        if (tok < 7) return 8;
        if (e == 0) {
            Rv[3 * blk] = rv[0];
            Rv[3 * blk + 1] = rv[1];
            Rv[3 * blk + 2] = rv[2];
        }
        const double w = (double)weights[(size_t)blk];
        double* o = &raw[2 * (size_t)(blk * NN + ind_j * nsta + ind_i)];
        o[0] = v[0] / w;
        o[1] = v[1] / w;
        return 0;
    });
    if (rc == -1) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _hr.dat is truncated");
    if (rc) {
        static const char* what[] = {"", "", "Missing R vector component", "Failed to parse R vector",
                                     "", "Failed to parse Hamiltonian real part",
                                     "Failed to parse Hamiltonian imaginary part",
                                     "Missing Hamiltonian real part", "Missing Hamiltonian imaginary part"};
        return file_error(file, what[rc]);
    }
    auto* h = new tbg_w90;
    h->nsta = nsta;
    h->weights = weights;
    h->hamR.assign(3, 0);
    h->ham.assign((size_t)NN * 2, 0.0);
    for (int64_t b = 0; b < nR; ++b) {
        const double* src = &raw[2 * (size_t)(b * NN)];
        if (Rv[3 * b] == 0 && Rv[3 * b + 1] == 0 && Rv[3 * b + 2] == 0) {
            std::copy(src, src + 2 * NN, h->ham.begin());
        } else {
            h->ham.insert(h->ham.end(), src, src + 2 * NN);
            h->hamR.insert(h->hamR.end(), {Rv[3 * b], Rv[3 * b + 1], Rv[3 * b + 2]});
        }
    }
    for (int64_t i = 0; i < nsta; ++i) h->ham[2 * (size_t)(i * nsta + i)] -= zero_energy;
    *out = h;
    return TBG_OK;
}

int tbg_w90_read_r(tbg_w90* h, const char* r_path) {
    if (!h || !r_path) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    const std::string file(r_path);
    std::string s;
    if (!read_file(r_path, s))
        return set_error(TBG_E_FILE_OPEN,
                         "Failed to create file '" + file + "': R::HAS_RMATRIX=true but _r.dat file not found");
    size_t pos = 0;
    std::vector<Line> head;
    for (int i = 0; i < 3 && pos < s.size(); ++i) head.push_back(line_at(s, pos));
    if (head.size() < 3) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _r.dat has fewer than 3 lines");
    int64_t nR = 0;
    const std::string u = trimmed(head[2]);
    if (!parse_u64(u.data(), u.data() + u.size(), nR))
        return file_error(file, "Failed to parse n_R: invalid digit found in string");
    const int64_t nsta = h->nsta, NN = nsta * nsta;
    if (nR > (int64_t)h->weights.size())
        return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _r.dat has more R vectors than _hr.dat weights");
    std::vector<double> raw((size_t)(nR * NN) * 6, 0.0);
    std::vector<int64_t> Rv((size_t)nR * 3, 0);
    const int rc = parallel_lines(s, pos, nR * NN, [&](int64_t L, Line l) -> int {
        const int64_t blk = L / NN, e = L % NN, ind_i = e / nsta, ind_j = e % nsta;
        const char* p = l.b;
        const char *tb, *te;
        double v[6];
        int tok = 0;
        int64_t rv[3];
        while (tok < 11 && next_token(p, l.e, tb, te)) {
            if (e == 0 && tok < 3 && !parse_i64(tb, te, rv[tok])) return 3;
            if (tok >= 5 && !parse_f64(tb, te, v[tok - 5])) return (tok - 5) % 2 == 0 ? 5 : 6;
            ++tok;
        }
        if (e == 0 && tok < 3) return 2;
        if (tok < 11) return (tok <= 5 || (tok - 5) % 2 == 0) ? 7 : 8;
        if (e == 0) {
            Rv[3 * blk] = rv[0];
            Rv[3 * blk + 1] = rv[1];
            Rv[3 * blk + 2] = rv[2];
        }
        const double w = (double)h->weights[(size_t)blk];
        for (int r = 0; r < 3; ++r) {
            double* o = &raw[2 * (size_t)(((blk * 3 + r) * nsta + ind_j) * nsta + ind_i)];
            o[0] = v[2 * r] / w;
            o[1] = v[2 * r + 1] / w;
        }
        return 0;
    });
    if (rc == -1) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _r.dat is truncated");
    if (rc) {
        static const char* what[] = {"", "", "Missing R vector component", "Failed to parse R vector",
                                     "", "Failed to parse R matrix real part",
                                     "Failed to parse R matrix imaginary part", "Missing R matrix real part",
                                     "Missing R matrix imaginary part"};
        return file_error(file, what[rc]);
    }
    const int64_t nRh = h->nR();
    h->rmat.assign((size_t)(nRh * 3 * NN) * 2, 0.0);
    for (int64_t b = 0; b < nR; ++b) {
        const int64_t idx = find_R(h->hamR, Rv[3 * b], Rv[3 * b + 1], Rv[3 * b + 2]);
        if (idx < 0) {
            char buf[160];
            std::snprintf(buf, sizeof(buf), "R vector [%lld, %lld, %lld] not found in Hamiltonian",
                          (long long)Rv[3 * b], (long long)Rv[3 * b + 1], (long long)Rv[3 * b + 2]);
            return file_error(file, buf);
        }
        const double* src = &raw[2 * (size_t)(b * 3 * NN)];
        std::copy(src, src + 6 * NN, h->rmat.begin() + 2 * (size_t)(idx * 3 * NN));
    }
    h->has_r = true;
    return TBG_OK;
}

int tbg_w90_apply_wsvec(tbg_w90* h, const char* ws_path, int* applied) {
    if (!h || !ws_path) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    if (applied) *applied = 0;
    const std::string file(ws_path);
    std::string s;
    if (!read_file(ws_path, s)) return TBG_OK;  // optional file
    std::vector<Line> lines;
    for (size_t pos = 0; pos < s.size();) lines.push_back(line_at(s, pos));
    if (lines.empty()) return set_error(TBG_E_INVALID_ARGUMENT, "attempt to subtract with overflow: empty _wsvec.dat");
    const int64_t nsta = h->nsta, NN = nsta * nsta;
    const bool R3 = h->has_r;
    std::vector<int64_t> nR_ = {0, 0, 0};
    std::vector<double> nham((size_t)NN * 2, 0.0), nrm(R3 ? (size_t)NN * 6 : 0, 0.0);
    auto bad = [&](const char* m) { return file_error(file, m); };
    size_t i = 0;
    while (i < lines.size() - 1) {
        ++i;
        const char* p = lines[i].b;
        const char *tb, *te;
        int64_t v[5];
        for (int t = 0; t < 5; ++t) {
            if (!next_token(p, lines[i].e, tb, te)) return bad(t < 3 ? "Missing R vector component" : "Missing orbital index");
            const bool ok = t < 3 ? parse_i64(tb, te, v[t]) : parse_u64(tb, te, v[t]);
            if (!ok) return bad(t < 3 ? "Failed to parse R vector" : "Failed to parse orbital index");
        }
        if (v[3] == 0 || v[4] == 0)
            return set_error(TBG_E_INVALID_ARGUMENT, "attempt to subtract with overflow (orbital index 0)");
        const int64_t oi = v[3] - 1, oj = v[4] - 1;
        if (oi >= nsta || oj >= nsta) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: orbital index");
        ++i;
        if (i >= lines.size()) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _wsvec.dat is truncated");
        p = lines[i].b;
        if (!next_token(p, lines[i].e, tb, te)) return bad("Missing weight value");
        int64_t weight = 0;
        if (!parse_u64(tb, te, weight)) return bad("Failed to parse weight");
        const int64_t idx = find_R(h->hamR, v[0], v[1], v[2]);
        if (idx < 0) {
            char buf[160];
            std::snprintf(buf, sizeof(buf), "R vector [%lld, %lld, %lld] not found in Hamiltonian", (long long)v[0],
                          (long long)v[1], (long long)v[2]);
            return bad(buf);
        }
        const size_t e = (size_t)(oi * nsta + oj);
        const double wd = (double)weight;
        const double hop_re = h->ham[2 * (idx * NN + e)] / wd, hop_im = h->ham[2 * (idx * NN + e) + 1] / wd;
        double rx[6] = {0, 0, 0, 0, 0, 0};
        if (R3)
            for (int r = 0; r < 3; ++r) {
                rx[2 * r] = h->rmat[2 * ((idx * 3 + r) * NN + e)] / wd;
                rx[2 * r + 1] = h->rmat[2 * ((idx * 3 + r) * NN + e) + 1] / wd;
            }
        for (int64_t k = 0; k < weight; ++k) {
            ++i;
            if (i >= lines.size()) return set_error(TBG_E_INVALID_ARGUMENT, "index out of bounds: _wsvec.dat is truncated");
            p = lines[i].b;
            int64_t T[3];
            for (int t = 0; t < 3; ++t)
                if (!next_token(p, lines[i].e, tb, te) || !parse_i64(tb, te, T[t]))
                    return set_error(TBG_E_INVALID_ARGUMENT, "called `Option::unwrap()` on a malformed shift line");
            const int64_t a = v[0] + T[0], b = v[1] + T[1], c = v[2] + T[2];
            int64_t j = find_R(nR_, a, b, c);
            if (j < 0) {
                j = (int64_t)nR_.size() / 3;
                nR_.insert(nR_.end(), {a, b, c});
                nham.resize(nham.size() + (size_t)NN * 2, 0.0);
                if (R3) nrm.resize(nrm.size() + (size_t)NN * 6, 0.0);
            }
            nham[2 * (j * NN + e)] += hop_re;
            nham[2 * (j * NN + e) + 1] += hop_im;
            if (R3)
                for (int r = 0; r < 3; ++r) {
                    nrm[2 * ((j * 3 + r) * NN + e)] += rx[2 * r];
                    nrm[2 * ((j * 3 + r) * NN + e) + 1] += rx[2 * r + 1];
                }
        }
    }
    h->hamR.swap(nR_);
    h->ham.swap(nham);
    if (R3) h->rmat.swap(nrm);
    if (applied) *applied = 1;
    return TBG_OK;
}

int tbg_w90_hermitize_rmatrix(tbg_w90* h) {
    if (!h) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    if (!h->has_r) return TBG_OK;
    const int64_t nsta = h->nsta, NN = nsta * nsta, nR = h->nR();
    double* m = h->rmat.data();
    for (int64_t r = 0; r + 1 < nR; ++r) {
        const int64_t* R = &h->hamR[3 * r];
        const int64_t q = find_R(h->hamR, -R[0], -R[1], -R[2]);
        if (q < 0) {
            char buf[160];
            std::snprintf(buf, sizeof(buf), "Missing Hermitian conjugate for R vector: [%lld, %lld, %lld]",
                          (long long)R[0], (long long)R[1], (long long)R[2]);
            return set_error(TBG_E_INVALID_MODEL, buf);
        }
        for (int64_t i = 0; i < nsta; ++i)
            for (int64_t j = 0; j < nsta; ++j)
                for (int c = 0; c < 3; ++c) {
                    double* a = m + 2 * ((r * 3 + c) * NN + i * nsta + j);
                    double* b = m + 2 * ((q * 3 + c) * NN + j * nsta + i);
                    const double re = (a[0] + b[0]) / 2.0, im = (a[1] - b[1]) / 2.0;
                    a[0] = re;
                    a[1] = im;
                    b[0] = re;
                    b[1] = -im;
                }
    }
    return TBG_OK;
}

int tbg_w90_info(const tbg_w90* h, int64_t* nsta, int64_t* nR, int* has_r) {
    if (!h) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    if (nsta) *nsta = h->nsta;
    if (nR) *nR = h->nR();
    if (has_r) *has_r = h->has_r ? 1 : 0;
    return TBG_OK;
}

int tbg_w90_copy(const tbg_w90* h, double* ham, int64_t* hamR, double* rmatrix) {
    if (!h) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    if (ham) std::copy(h->ham.begin(), h->ham.end(), ham);
    if (hamR) std::copy(h->hamR.begin(), h->hamR.end(), hamR);
    if (rmatrix && h->has_r) std::copy(h->rmat.begin(), h->rmat.end(), rmatrix);
    return TBG_OK;
}

int tbg_w90_free(tbg_w90* h) {
    delete h;
    return TBG_OK;
}

}  // extern "C"

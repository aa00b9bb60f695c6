// MPS ingest for the engine: a file (or an in-memory text) to the CSC and CSR
// arrays of sih_pdhg_problem in one pass over the text.
//
// Record semantics are the reference reader's (core/src/io/mps_io.cpp:63-323),
// so a file gives the same problem through either reader:
//   - lines that start with '*' are comments; a line whose first character is
//     not white space is a section header (NAME, OBJSENSE, ROWS, COLUMNS, RHS,
//     RANGES, BOUNDS, QUADOBJ, QMATRIX, ENDATA; any other header is skipped
//     and leaves the current section as it was);
//   - records are split at white space outside apostrophes;
//   - the first N row is the objective; further N rows and entries of unknown
//     rows are dropped; a repeated row name keeps its first definition;
//   - COLUMNS: column, then (row, value) pairs; 'MARKER' 'INTORG' / 'INTEND'
//     mark integer columns (the PDHG solve takes the LP relaxation);
//   - RHS / RANGES: an odd token count means a leading set name; the objective
//     row's RHS sets obj_offset = -value (the last one wins);
//   - BOUNDS: type, set name, column [, value (0 if absent)]; UP LO FX FR MI
//     (lower -inf, upper 0) PL BV UI LI; a bound may create a column;
//   - row bounds from type and RHS, with |R| on G / L rows and the sign of R on
//     E rows; rows of another type stay free;
//   - duplicate (row, column) entries are summed in file order and entries
//     with |value| <= 1e-15 dropped (SparseMatrix::from_triplets,
//     core/src/model/sparse_matrix.cpp:13-88); contradictory row or column
//     bounds are an error (Problem::validate, core/src/model/problem.cpp:117-150);
//   - numbers are read as std::stod reads them: leading part of the token,
//     an error when nothing converts or the value is out of range.
// Differences: errors are status codes with the line number instead of C++
// exceptions, and a QUADOBJ / QMATRIX section is rejected (this engine solves
// LPs).  The matrix is built by counting sorts over the entries rather than an
// ordered coordinate map.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#include <sys/stat.h>

#include "sih_pdhg.h"

namespace sihg {
void set_last_error(const std::string& msg);
}

struct sih_pdhg_mps {
    std::string name = "problem";  // sih::model::Problem's default name (problem.hpp:113)
    int64_t m = 0, n = 0, nnz = 0;
    std::vector<int64_t> csc_ptr, csc_row, csr_ptr, csr_col;
    std::vector<double> csc_val, csr_val, c, col_lower, col_upper, row_lower, row_upper;
    int32_t sense = 1;
    double obj_offset = 0.0;
    int64_t integer_columns = 0;
};

namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr double kZeroTol = 1e-15;

enum class Sec { None, Name, ObjSense, Rows, Columns, Rhs, Ranges, Bounds, Quad, End };

struct ParseError {
    std::string msg;
};

// std::isspace in the C locale: space, \t, \n, \v, \f, \r.
inline bool is_space(char ch) { return ch == ' ' || (ch >= '\t' && ch <= '\r'); }

std::string upper(std::string_view s) {
    std::string out(s);
    for (auto& ch : out) ch = (char)std::toupper(static_cast<unsigned char>(ch));
    return out;
}

// Section of a header keyword, or Sec::None for a header line the reader skips.
Sec header_section(std::string_view first_token) {
    const std::string h = upper(first_token);
    if (h == "NAME") return Sec::Name;
    if (h == "OBJSENSE") return Sec::ObjSense;
    if (h == "ROWS") return Sec::Rows;
    if (h == "COLUMNS") return Sec::Columns;
    if (h == "RHS") return Sec::Rhs;
    if (h == "RANGES") return Sec::Ranges;
    if (h == "BOUNDS") return Sec::Bounds;
    if (h == "QUADOBJ" || h == "QMATRIX") return Sec::Quad;
    if (h == "ENDATA") return Sec::End;
    return Sec::None;
}

// White-space separated tokens; apostrophes toggle quoting and stay in the token.
int tokenize(std::string_view line, std::vector<std::string_view>& tok) {
    tok.clear();
    bool quoted = false;
    size_t start = std::string_view::npos;
    for (size_t i = 0; i < line.size(); ++i) {
        const char ch = line[i];
        if (ch == '\'') {
            quoted = !quoted;
            if (start == std::string_view::npos) start = i;
        } else if (is_space(ch) && !quoted) {
            if (start != std::string_view::npos) {
                tok.push_back(line.substr(start, i - start));
                start = std::string_view::npos;
            }
        } else if (start == std::string_view::npos) {
            start = i;
        }
    }
    if (start != std::string_view::npos) tok.push_back(line.substr(start));
    return (int)tok.size();
}

// A plain decimal token ([-]digits[.digits][e[+-]digits], all of it): the
// correctly rounded value that strtod also gives, without the locale work.
bool plain_decimal(std::string_view t) {
    size_t i = 0, n = t.size();
    if (i < n && t[i] == '-') ++i;
    size_t d = 0;
    while (i < n && t[i] >= '0' && t[i] <= '9') ++i, ++d;
    if (i < n && t[i] == '.') {
        ++i;
        while (i < n && t[i] >= '0' && t[i] <= '9') ++i, ++d;
    }
    if (d == 0) return false;
    if (i < n && (t[i] == 'e' || t[i] == 'E')) {
        ++i;
        if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
        size_t e = 0;
        while (i < n && t[i] >= '0' && t[i] <= '9') ++i, ++e;
        if (e == 0) return false;
    }
    return i == n;
}

// A token that std::stod would reject (nothing converts, or out of range).
struct NumberError {
    std::string token;
    bool out_of_range;
};

double number_value(std::string_view t) {
    if (plain_decimal(t)) {
        double v = 0.0;
        const auto r = std::from_chars(t.data(), t.data() + t.size(), v);
        if (r.ec == std::errc() && r.ptr == t.data() + t.size()) return v;
        // out of range: strtod below reports it as std::stod would
    }
    char buf[128];
    std::string big;
    const char* s;
    if (t.size() < sizeof(buf)) {
        std::memcpy(buf, t.data(), t.size());
        buf[t.size()] = '\0';
        s = buf;
    } else {
        big.assign(t);
        s = big.c_str();
    }
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(s, &end);
    if (end == s) throw NumberError{std::string(t), false};
    if (errno == ERANGE) throw NumberError{std::string(t), true};
    return v;
}

std::string number_message(int64_t line_no, const NumberError& e) {
    return "line " + std::to_string(line_no) + ": '" + e.token + (e.out_of_range ? "' is out of range"
                                                                                  : "' is not a number");
}

double number(std::string_view t, int64_t line_no) {
    try {
        return number_value(t);
    } catch (const NumberError& e) {
        throw ParseError{number_message(line_no, e)};
    }
}

struct RowDef {
    char type;
    double rhs = 0.0, range = 0.0;
    bool has_range = false;
};

// Name -> index, open addressing over a flat slot array: one probe touches one
// 24-byte slot, and the stored hash rejects other names without reading them
// (row and column names of a large file are looked up millions of times).
class NameTable {
    struct Slot {
        uint64_t h;
        const char* p;
        uint32_t len;
        int32_t val;  // -1 = empty
    };
    std::vector<Slot> slots_;
    size_t mask_ = 0, count_ = 0;

    static uint64_t hash(std::string_view s) {
        uint64_t h = 1469598103934665603ull;  // FNV-1a, then a multiplicative finaliser
        for (unsigned char ch : s) h = (h ^ ch) * 1099511628211ull;
        h ^= h >> 29;
        h *= 0xbf58476d1ce4e5b9ull;
        return h ^ (h >> 32);
    }
    void grow() {
        std::vector<Slot> old;
        old.swap(slots_);
        const size_t cap = old.empty() ? 1024 : old.size() * 2;
        slots_.assign(cap, Slot{0, nullptr, 0, -1});
        mask_ = cap - 1;
        for (const Slot& s : old)
            if (s.val >= 0) place(s);
    }
    void place(const Slot& s) {
        size_t i = s.h & mask_;
        while (slots_[i].val >= 0) i = (i + 1) & mask_;
        slots_[i] = s;
    }

   public:
    // Index of `name`, or -1.
    int64_t find(std::string_view name) const {
        if (slots_.empty()) return -1;
        const uint64_t h = hash(name);
        for (size_t i = h & mask_;; i = (i + 1) & mask_) {
            const Slot& s = slots_[i];
            if (s.val < 0) return -1;
            if (s.h == h && s.len == name.size() && std::memcmp(s.p, name.data(), name.size()) == 0) return s.val;
        }
    }
    // Adds name -> val (the caller has checked that the name is new).
    void insert(std::string_view name, int64_t val) {
        if (val > std::numeric_limits<int32_t>::max() || name.size() > std::numeric_limits<uint32_t>::max())
            throw ParseError{"more than 2^31 - 1 rows or columns"};
        if (2 * (count_ + 1) > slots_.size()) grow();
        place(Slot{hash(name), name.data(), (uint32_t)name.size(), (int32_t)val});
        ++count_;
    }
};

// COLUMNS bodies of at least this many bytes are parsed on several threads
// (environment SIH_PDHG_MPS_PARALLEL_BYTES overrides; 0 = always).
size_t parallel_min_bytes() {
    if (const char* v = std::getenv("SIH_PDHG_MPS_PARALLEL_BYTES")) {
        char* end = nullptr;
        const long long n = std::strtoll(v, &end, 10);
        if (end != v && n >= 0) return (size_t)n;
    }
    return (size_t)8 << 20;
}

struct Reader {
    sih_pdhg_mps& P;
    NameTable row_index;
    std::vector<RowDef> rows;
    std::vector<std::string_view> row_order;
    std::string_view obj_row;
    bool have_obj = false;
    NameTable cols;
    std::string_view last_col;
    int64_t last_col_idx = -1;
    std::vector<char> col_int;
    std::vector<int64_t> e_row, e_col;
    std::vector<double> e_val;
    bool integer_marker = false, quadratic = false;

    explicit Reader(sih_pdhg_mps& p) : P(p) {}

    // A new column as the reference creates one: c 0, bounds [0, +inf).
    int64_t create_column(std::string_view name, bool integer) {
        const int64_t idx = (int64_t)P.c.size();
        cols.insert(name, idx);
        col_int.push_back(integer ? 1 : 0);
        P.col_lower.push_back(0.0);
        P.col_upper.push_back(kInf);
        P.c.push_back(0.0);
        return idx;
    }

    int64_t column(std::string_view name) {
        if (last_col_idx >= 0 && name == last_col) return last_col_idx;
        int64_t idx = cols.find(name);
        if (idx < 0) idx = create_column(name, integer_marker);
        last_col = name;
        last_col_idx = idx;
        return idx;
    }

    // End of the COLUMNS body that starts at `pos`: the start of the next line
    // with a section keyword (other header lines are skipped and stay inside).
    static size_t columns_end(std::string_view text, size_t pos) {
        std::vector<std::string_view> tok;
        while (pos < text.size()) {
            size_t eol = text.find('\n', pos);
            if (eol == std::string_view::npos) eol = text.size();
            const std::string_view line = text.substr(pos, eol - pos);
            if (!line.empty() && line[0] != '*' && !is_space(line[0]) && tokenize(line, tok) > 0 &&
                header_section(tok[0]) != Sec::None)
                return pos;
            pos = eol + 1;
        }
        return text.size();
    }

    // One slice of a COLUMNS body, parsed on its own thread: columns first seen
    // here (with the integer marker state at that point, -1 = the state the
    // slice starts with), entries and objective terms by local column, in file
    // order, and the slice's first number error.
    struct ColSlice {
        NameTable local;
        std::vector<std::string_view> names;
        std::vector<signed char> name_marker;
        std::vector<int32_t> e_lcol, obj_lcol;
        std::vector<int64_t> e_row;
        std::vector<double> e_val, obj_val;
        signed char final_marker = -1;
        bool failed = false;
        size_t fail_line = 0;  // byte offset of the failing line
        NumberError error{std::string(), false};
    };

    void parse_slice(std::string_view text, size_t b, size_t e, ColSlice& S) const {
        std::vector<std::string_view> tok;
        tok.reserve(16);
        signed char marker = -1;
        std::string_view last;
        int32_t last_id = -1;
        size_t pos = b;
        while (pos < e) {
            size_t eol = text.find('\n', pos);
            if (eol == std::string_view::npos || eol > e) eol = e;
            const std::string_view line = text.substr(pos, eol - pos);
            const size_t line_start = pos;
            pos = eol + 1;
            if (line.empty() || line[0] == '*' || !is_space(line[0])) continue;  // comment, skipped header
            const int nt = tokenize(line, tok);
            if (nt >= 3 && (tok[1] == "'MARKER'" || tok[1] == "MARKER")) {
                const std::string mk = upper(tok[2]);
                if (mk == "'INTORG'" || mk == "INTORG") marker = 1;
                else if (mk == "'INTEND'" || mk == "INTEND") marker = 0;
                continue;
            }
            if (nt < 3) continue;
            int32_t id = last_id;
            if (id < 0 || tok[0] != last) {
                int64_t f = S.local.find(tok[0]);
                if (f < 0) {
                    f = (int64_t)S.names.size();
                    S.local.insert(tok[0], f);
                    S.names.push_back(tok[0]);
                    S.name_marker.push_back(marker);
                }
                id = (int32_t)f;
                last = tok[0];
                last_id = id;
            }
            for (int k = 1; k + 1 < nt; k += 2) {
                double v;
                try {
                    v = number_value(tok[k + 1]);
                } catch (const NumberError& err) {
                    S.failed = true;
                    S.fail_line = line_start;
                    S.error = err;
                    return;
                }
                if (have_obj && tok[k] == obj_row) {
                    S.obj_lcol.push_back(id);
                    S.obj_val.push_back(v);
                } else {
                    const int64_t i = row_index.find(tok[k]);
                    if (i >= 0) {
                        S.e_lcol.push_back(id);
                        S.e_row.push_back(i);
                        S.e_val.push_back(v);
                    }
                }
            }
        }
        S.final_marker = marker;
    }

    // The COLUMNS body [b, e) on several threads, merged in file order: the
    // same columns (first appearance order, marker state), entries and
    // objective sums as a sequential pass, and the first number error of the
    // file.  `line_no` is the number of the COLUMNS header line.
    void parse_columns_parallel(std::string_view text, size_t b, size_t e, int64_t line_no) {
        int T = (int)std::thread::hardware_concurrency();
        T = std::max(2, std::min(T, 32));
        std::vector<size_t> cut(T + 1, b);
        cut[T] = e;
        for (int k = 1; k < T; ++k) {
            size_t q = b + (size_t)((double)(e - b) * k / T);
            if (q > b) {
                const size_t nl = text.find('\n', q - 1);
                q = (nl == std::string_view::npos || nl + 1 > e) ? e : nl + 1;
            }
            cut[k] = std::max(cut[k - 1], std::min(q, e));
        }
        std::vector<ColSlice> slices(T);
        std::vector<std::thread> pool;
        for (int k = 0; k < T; ++k)
            pool.emplace_back([&, k] { parse_slice(text, cut[k], cut[k + 1], slices[k]); });
        for (auto& t : pool) t.join();
        for (const ColSlice& S : slices)
            if (S.failed) {
                const int64_t line = line_no + 1 + std::count(text.begin() + b, text.begin() + S.fail_line, '\n');
                throw ParseError{number_message(line, S.error)};
            }
        bool state = integer_marker;
        for (const ColSlice& S : slices) {
            std::vector<int64_t> map(S.names.size());
            for (size_t t = 0; t < S.names.size(); ++t) {
                int64_t g = cols.find(S.names[t]);
                if (g < 0) g = create_column(S.names[t], S.name_marker[t] >= 0 ? S.name_marker[t] == 1 : state);
                map[t] = g;
            }
            if (S.final_marker >= 0) state = S.final_marker == 1;
            for (size_t q = 0; q < S.obj_lcol.size(); ++q) P.c[map[S.obj_lcol[q]]] += S.obj_val[q];
            for (size_t q = 0; q < S.e_lcol.size(); ++q) {
                e_row.push_back(S.e_row[q]);
                e_col.push_back(map[S.e_lcol[q]]);
                e_val.push_back(S.e_val[q]);
            }
        }
        integer_marker = state;
        last_col_idx = -1;
    }

    void parse(std::string_view text) {
        Sec sec = Sec::None;
        std::vector<std::string_view> tok;
        tok.reserve(16);
        int64_t line_no = 0;
        size_t pos = 0;
        while (pos < text.size()) {
            size_t eol = text.find('\n', pos);
            if (eol == std::string_view::npos) eol = text.size();
            const std::string_view line = text.substr(pos, eol - pos);
            pos = eol + 1;
            ++line_no;
            if (line.empty() || line[0] == '*') continue;
            if (!is_space(line[0])) {
                if (tokenize(line, tok) == 0) continue;
                const Sec h = header_section(tok[0]);
                if (h == Sec::None) continue;  // a header the reference skips: the section stays
                if (h == Sec::End) return;
                sec = h;
                if (h == Sec::Name && tok.size() > 1) P.name.assign(tok[1]);
                if (h == Sec::Columns) {
                    const size_t body_end = columns_end(text, pos);
                    if (body_end - std::min(pos, body_end) >= parallel_min_bytes()) {
                        parse_columns_parallel(text, pos, body_end, line_no);
                        line_no += std::count(text.begin() + pos, text.begin() + body_end, '\n');
                        pos = body_end;
                    }
                }
                continue;
            }
            const int nt = tokenize(line, tok);
            if (nt == 0) continue;
            switch (sec) {
                case Sec::ObjSense: {
                    const std::string s = upper(tok[0]);
                    if (s == "MAX" || s == "MAXIMIZE") P.sense = -1;
                    else if (s == "MIN" || s == "MINIMIZE") P.sense = 1;
                    break;
                }
                case Sec::Rows: {
                    if (nt < 2) break;
                    const char type = (char)std::toupper(static_cast<unsigned char>(tok[0][0]));
                    if (type == 'N') {
                        if (!have_obj) {
                            obj_row = tok[1];
                            have_obj = true;
                        }
                    } else if (row_index.find(tok[1]) < 0) {
                        row_index.insert(tok[1], (int64_t)row_order.size());
                        rows.push_back(RowDef{type});
                        row_order.push_back(tok[1]);
                    }
                    break;
                }
                case Sec::Columns: {
                    if (nt >= 3 && (tok[1] == "'MARKER'" || tok[1] == "MARKER")) {
                        const std::string mk = upper(tok[2]);
                        if (mk == "'INTORG'" || mk == "INTORG") integer_marker = true;
                        else if (mk == "'INTEND'" || mk == "INTEND") integer_marker = false;
                        break;
                    }
                    if (nt < 3) break;
                    const int64_t j = column(tok[0]);
                    for (int k = 1; k + 1 < nt; k += 2) {
                        const double v = number(tok[k + 1], line_no);
                        if (have_obj && tok[k] == obj_row) {
                            P.c[j] += v;
                        } else {
                            const int64_t i = row_index.find(tok[k]);
                            if (i >= 0) {
                                e_row.push_back(i);
                                e_col.push_back(j);
                                e_val.push_back(v);
                            }
                        }
                    }
                    break;
                }
                case Sec::Rhs:
                case Sec::Ranges: {
                    for (int k = (nt % 2 == 1) ? 1 : 0; k + 1 < nt; k += 2) {
                        const double v = number(tok[k + 1], line_no);
                        if (sec == Sec::Rhs && have_obj && tok[k] == obj_row) {
                            P.obj_offset = -v;
                            continue;
                        }
                        const int64_t i = row_index.find(tok[k]);
                        if (i < 0) continue;
                        if (sec == Sec::Rhs) {
                            rows[i].rhs = v;
                        } else {
                            rows[i].range = v;
                            rows[i].has_range = true;
                        }
                    }
                    break;
                }
                case Sec::Bounds: {
                    if (nt < 3) break;
                    const std::string bt = upper(tok[0]);
                    const double v = nt >= 4 ? number(tok[3], line_no) : 0.0;
                    const int64_t j = column(tok[2]);
                    double& lo = P.col_lower[j];
                    double& up = P.col_upper[j];
                    if (bt == "UP") up = v;
                    else if (bt == "LO") lo = v;
                    else if (bt == "FX") lo = up = v;
                    else if (bt == "FR") { lo = -kInf; up = kInf; }
                    else if (bt == "MI") { lo = -kInf; up = 0.0; }
                    else if (bt == "PL") { lo = 0.0; up = kInf; }
                    else if (bt == "BV") { col_int[j] = 1; lo = 0.0; up = 1.0; }
                    else if (bt == "UI") { col_int[j] = 1; up = v; }
                    else if (bt == "LI") { col_int[j] = 1; lo = v; }
                    break;
                }
                case Sec::Quad: {
                    if (nt < 3) break;
                    number(tok[2], line_no);
                    column(tok[0]);
                    column(tok[1]);
                    quadratic = true;
                    break;
                }
                default:
                    break;
            }
        }
    }

    void finish() {
        const int64_t m = (int64_t)row_order.size(), n = (int64_t)P.c.size();
        P.m = m;
        P.n = n;
        P.row_lower.assign(m, -kInf);
        P.row_upper.assign(m, kInf);
        for (int64_t i = 0; i < m; ++i) {
            const RowDef& r = rows[i];
            double& lo = P.row_lower[i];
            double& up = P.row_upper[i];
            if (!r.has_range) {
                if (r.type == 'G') { lo = r.rhs; up = kInf; }
                else if (r.type == 'L') { lo = -kInf; up = r.rhs; }
                else if (r.type == 'E') { lo = up = r.rhs; }
            } else {
                const double a = std::fabs(r.range);
                if (r.type == 'G') { lo = r.rhs; up = r.rhs + a; }
                else if (r.type == 'L') { lo = r.rhs - a; up = r.rhs; }
                else if (r.type == 'E') {
                    if (r.range >= 0.0) { lo = r.rhs; up = r.rhs + r.range; }
                    else { lo = r.rhs + r.range; up = r.rhs; }
                }
            }
        }
        for (char f : col_int) P.integer_columns += f;
        for (int64_t i = 0; i < m; ++i)
            if (P.row_lower[i] > P.row_upper[i])
                throw ParseError{"contradictory row bounds at row " + std::to_string(i) + " (" +
                                 std::string(row_order[i]) + ")"};
        for (int64_t j = 0; j < n; ++j)
            if (P.col_lower[j] > P.col_upper[j])
                throw ParseError{"contradictory column bounds at column " + std::to_string(j)};
        build_matrix();
    }

    // CSC: entries bucketed by column in file order (counting sort), each
    // column ordered by row (stable, so duplicates keep file order), duplicates
    // summed in that order, |sum| <= 1e-15 dropped.  CSR: a counting sort of
    // the CSC by row, which leaves columns ascending within each row.
    void build_matrix() {
        const int64_t n = P.n, m = P.m, E = (int64_t)e_val.size();
        std::vector<int64_t> ptr(n + 1, 0);
        for (int64_t k = 0; k < E; ++k) ptr[e_col[k] + 1]++;
        for (int64_t j = 0; j < n; ++j) ptr[j + 1] += ptr[j];
        std::vector<int64_t> order(E), fill(ptr.begin(), ptr.end() - 1);
        for (int64_t k = 0; k < E; ++k) order[fill[e_col[k]]++] = k;
        P.csc_ptr.assign(n + 1, 0);
        P.csc_row.clear();
        P.csc_val.clear();
        P.csc_row.reserve(E);
        P.csc_val.reserve(E);
        for (int64_t j = 0; j < n; ++j) {
            auto b = order.begin() + ptr[j], e = order.begin() + ptr[j + 1];
            bool sorted = true;
            for (auto it = b; it + 1 < e; ++it)
                if (e_row[*(it + 1)] < e_row[*it]) { sorted = false; break; }
            if (!sorted) std::stable_sort(b, e, [&](int64_t x, int64_t y) { return e_row[x] < e_row[y]; });
            for (auto it = b; it < e;) {
                const int64_t r = e_row[*it];
                double s = e_val[*it];
                for (++it; it < e && e_row[*it] == r; ++it) s += e_val[*it];
                if (std::fabs(s) > kZeroTol) {
                    P.csc_row.push_back(r);
                    P.csc_val.push_back(s);
                }
            }
            P.csc_ptr[j + 1] = (int64_t)P.csc_row.size();
        }
        P.nnz = (int64_t)P.csc_row.size();
        P.csr_ptr.assign(m + 1, 0);
        for (int64_t k = 0; k < P.nnz; ++k) P.csr_ptr[P.csc_row[k] + 1]++;
        for (int64_t i = 0; i < m; ++i) P.csr_ptr[i + 1] += P.csr_ptr[i];
        P.csr_col.resize(P.nnz);
        P.csr_val.resize(P.nnz);
        std::vector<int64_t> rf(P.csr_ptr.begin(), P.csr_ptr.end() - 1);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t k = P.csc_ptr[j]; k < P.csc_ptr[j + 1]; ++k) {
                const int64_t d = rf[P.csc_row[k]]++;
                P.csr_col[d] = j;
                P.csr_val[d] = P.csc_val[k];
            }
    }
};

int read_text(std::string_view text, sih_pdhg_mps** out) {
    auto* P = new (std::nothrow) sih_pdhg_mps();
    if (!P) {
        sihg::set_last_error("out of host memory");
        return SIH_PDHG_ERR_OUT_OF_MEMORY;
    }
    try {
        Reader R(*P);
        R.parse(text);
        if (R.quadratic) {
            delete P;
            sihg::set_last_error("the file has a quadratic objective (QUADOBJ / QMATRIX); this engine solves LPs");
            return SIH_PDHG_ERR_UNSUPPORTED;
        }
        R.finish();
    } catch (const ParseError& e) {
        delete P;
        sihg::set_last_error("MPS: " + e.msg);
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    } catch (const std::bad_alloc&) {
        delete P;
        sihg::set_last_error("MPS: out of host memory");
        return SIH_PDHG_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {  // nothing may cross the C boundary
        delete P;
        sihg::set_last_error(std::string("MPS: ") + e.what());
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    *out = P;
    return SIH_PDHG_OK;
}

}  // namespace

extern "C" {

int sih_pdhg_read_mps_text(const char* text, size_t length, sih_pdhg_mps** out) {
    if (!out || (!text && length > 0)) {
        sihg::set_last_error("NULL argument");
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    return read_text(std::string_view(text ? text : "", length), out);
}

int sih_pdhg_read_mps(const char* path, sih_pdhg_mps** out) {
    if (!path || !out) {
        sihg::set_last_error("NULL argument");
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) {
        sihg::set_last_error(std::string("could not open MPS file: ") + path);
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    std::string text;
    char buf[1 << 16];
    size_t got;
    try {
        // a directory is an error; a regular file is read into one allocation of
        // its size; anything else (a pipe, a device) is read to its end
        struct stat st;
        const bool have_stat = fstat(fileno(f), &st) == 0;
        if (have_stat && S_ISDIR(st.st_mode)) {
            std::fclose(f);
            sihg::set_last_error(std::string("is a directory: ") + path);
            return SIH_PDHG_ERR_INVALID_ARGUMENT;
        }
        if (have_stat && S_ISREG(st.st_mode) && st.st_size > 0) text.reserve((size_t)st.st_size);
        while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    } catch (const std::exception&) {
        std::fclose(f);
        sihg::set_last_error("MPS: out of host memory");
        return SIH_PDHG_ERR_OUT_OF_MEMORY;
    }
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    if (bad) {
        sihg::set_last_error(std::string("error reading MPS file: ") + path);
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    return read_text(text, out);
}

int sih_pdhg_mps_view(const sih_pdhg_mps* mps, sih_pdhg_problem* problem, const char** name,
                      int64_t* integer_columns) {
    if (!mps || !problem) {
        sihg::set_last_error("NULL argument");
        return SIH_PDHG_ERR_INVALID_ARGUMENT;
    }
    problem->num_rows = mps->m;
    problem->num_cols = mps->n;
    problem->num_nonzeros = mps->nnz;
    problem->csc_col_ptr = mps->csc_ptr.data();
    problem->csc_row_ind = mps->csc_row.data();
    problem->csc_values = mps->csc_val.data();
    problem->csr_row_ptr = mps->csr_ptr.data();
    problem->csr_col_ind = mps->csr_col.data();
    problem->csr_values = mps->csr_val.data();
    problem->c = mps->c.data();
    problem->col_lower = mps->col_lower.data();
    problem->col_upper = mps->col_upper.data();
    problem->row_lower = mps->row_lower.data();
    problem->row_upper = mps->row_upper.data();
    problem->sense = mps->sense;
    problem->obj_offset = mps->obj_offset;
    if (name) *name = mps->name.c_str();
    if (integer_columns) *integer_columns = mps->integer_columns;
    return SIH_PDHG_OK;
}

void sih_pdhg_mps_free(sih_pdhg_mps* mps) { delete mps; }

}  // extern "C"

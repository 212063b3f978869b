// acdalm_read_mps: an LP in (free-format) MPS, turned into the solver's
// form  min c'x  s.t.  A x = b,  l <= x <= u.
//
// Every constraint row i of the file is a_i x (<=, >=, =) rhs_i, possibly
// with a RANGES entry.  Equality rows without a range stay equalities.  Any
// other row r gets a slack column s_r, its coefficient -1 in that row:
// a_r x - s_r = 0, with the row's interval [lo_r, hi_r] as the slack's
// bounds (L: (-inf, rhs], G: [rhs, +inf), ranged rows: the MPS range
// rules).  Multiplier bounds are free.  Columns keep their order of first
// appearance; slack columns follow, in row order.  The first N row is the
// objective; OBJSENSE MAX negates it.  Integer markers are ignored (the
// relaxation is solved).  Bound types: UP, LO, FX, FR, MI, PL, BV (a
// negative UP on a column whose lower bound is still the default 0 sets
// the lower bound to -inf, the usual MPS convention).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/acdalm_ext.h"
#include "../../include/alm.h"
#include "../../include/spmv.h"
#include "common.h"

namespace {

struct Row {
        char type;  // 'N', 'L', 'G', 'E'
        double rhs = 0;
        bool ranged = false;
        double range = 0;
};

struct Entry {
        uint32_t row, col;
        double val;
};

std::vector<std::string> tokens(const char * line)
{
        std::vector<std::string> t;
        const char * p = line;
        while (*p) {
                while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')
                        p++;
                if (!*p)
                        break;
                const char * q = p;
                while (*q && *q != ' ' && *q != '\t' && *q != '\r' && *q != '\n')
                        q++;
                t.emplace_back(p, q - p);
                p = q;
        }
        return t;
}

bool number(const std::string & s, double & v)
{
        char * end = nullptr;
        v = strtod(s.c_str(), &end);
        return end && *end == '\0' && !s.empty();
}

struct Parser {
        std::vector<Row> rows;  // constraint rows (N rows kept apart)
        std::unordered_map<std::string, int> row_of;  // >= 0 constraint, -1 objective, -2 other N
        std::vector<std::string> col_names;
        std::unordered_map<std::string, uint32_t> col_of;
        std::vector<double> cost, lower, upper;
        std::vector<bool> lower_set;
        std::vector<Entry> entries;
        bool have_objective = false;
        bool maximize = false;
        int line_no = 0;

        bool fail(const char * what)
        {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_mps: line %d: %s", line_no, what);
                return false;
        }

        uint32_t column(const std::string & name)
        {
                auto it = col_of.find(name);
                if (it != col_of.end())
                        return it->second;
                uint32_t j = (uint32_t)col_names.size();
                col_of.emplace(name, j);
                col_names.push_back(name);
                cost.push_back(0);
                lower.push_back(0);
                upper.push_back(HUGE_VAL);
                lower_set.push_back(false);
                return j;
        }

        bool row_decl(const std::vector<std::string> & t)
        {
                if (t.size() != 2 || t[0].size() != 1)
                        return fail("ROWS entries are: type name");
                char type = t[0][0];
                if (type == 'N') {
                        row_of[t[1]] = have_objective ? -2 : -1;
                        have_objective = true;
                        return true;
                }
                if (type != 'L' && type != 'G' && type != 'E')
                        return fail("row type must be N, L, G or E");
                if (row_of.count(t[1]))
                        return fail("duplicate row name");
                row_of[t[1]] = (int)rows.size();
                Row r;
                r.type = type;
                rows.push_back(r);
                return true;
        }

        bool coefficient(uint32_t j, const std::string & row, const std::string & val)
        {
                double v;
                if (!number(val, v))
                        return fail("bad number");
                auto it = row_of.find(row);
                if (it == row_of.end())
                        return fail("unknown row");
                if (it->second == -1)
                        cost[j] += v;
                else if (it->second >= 0 && v != 0)
                        entries.push_back({(uint32_t)it->second, j, v});
                return true;
        }

        bool columns(const std::vector<std::string> & t)
        {
                if (t.size() >= 2 && t[1] == "'MARKER'")
                        return true;
                if (t.size() != 3 && t.size() != 5)
                        return fail("COLUMNS entries are: column row value [row value]");
                uint32_t j = column(t[0]);
                for (size_t k = 1; k + 1 < t.size(); k += 2)
                        if (!coefficient(j, t[k], t[k + 1]))
                                return false;
                return true;
        }

        // RHS and RANGES: [set] row value [row value]
        bool row_values(const std::vector<std::string> & t, bool range)
        {
                size_t first = (t.size() % 2 == 1) ? 1 : 0;
                if (t.size() < 2 || t.size() > 5)
                        return fail("RHS / RANGES entries are: [set] row value [row value]");
                for (size_t k = first; k + 1 < t.size(); k += 2) {
                        double v;
                        if (!number(t[k + 1], v))
                                return fail("bad number");
                        auto it = row_of.find(t[k]);
                        if (it == row_of.end())
                                return fail("unknown row");
                        if (it->second < 0)
                                continue;  // objective constant / free rows: ignored
                        Row & r = rows[it->second];
                        if (range) {
                                r.ranged = true;
                                r.range = v;
                        } else {
                                r.rhs = v;
                        }
                }
                return true;
        }

        bool bound(const std::vector<std::string> & t)
        {
                if (t.empty())
                        return true;
                const std::string & type = t[0];
                bool valueless = type == "FR" || type == "MI" || type == "PL" || type == "BV";
                size_t need = valueless ? 2 : 3;
                if (t.size() != need && t.size() != need + 1)
                        return fail("BOUNDS entries are: type [set] column [value]");
                size_t ci = (t.size() == need + 1) ? 2 : 1;
                auto it = col_of.find(t[ci]);
                if (it == col_of.end())
                        return fail("unknown column");
                uint32_t j = it->second;
                double v = 0;
                if (!valueless && !number(t[ci + 1], v))
                        return fail("bad number");
                if (type == "UP") {
                        upper[j] = v;
                        if (v < 0 && !lower_set[j] && lower[j] == 0)
                                lower[j] = -HUGE_VAL;
                } else if (type == "LO") {
                        lower[j] = v;
                        lower_set[j] = true;
                } else if (type == "FX") {
                        lower[j] = upper[j] = v;
                        lower_set[j] = true;
                } else if (type == "FR") {
                        lower[j] = -HUGE_VAL;
                        upper[j] = HUGE_VAL;
                } else if (type == "MI") {
                        lower[j] = -HUGE_VAL;
                        lower_set[j] = true;
                } else if (type == "PL") {
                        upper[j] = HUGE_VAL;
                } else if (type == "BV") {
                        lower[j] = 0;
                        upper[j] = 1;
                        lower_set[j] = true;
                } else {
                        return fail("bound type must be UP, LO, FX, FR, MI, PL or BV");
                }
                return true;
        }

        bool parse(FILE * f)
        {
                enum { NONE, NAME, ROWS, COLUMNS, RHS, RANGES, BOUNDS, OBJSENSE, END } sec = NONE;
                std::vector<char> buf(1 << 16);
                while (fgets(buf.data(), (int)buf.size(), f)) {
                        line_no++;
                        const char * line = buf.data();
                        if (line[0] == '*' || line[0] == '\n' || line[0] == '\r' || line[0] == '\0')
                                continue;
                        std::vector<std::string> t = tokens(line);
                        if (t.empty())
                                continue;
                        if (line[0] != ' ' && line[0] != '\t') {
                                const std::string & h = t[0];
                                if (h == "NAME")
                                        sec = NAME;
                                else if (h == "ROWS")
                                        sec = ROWS;
                                else if (h == "COLUMNS")
                                        sec = COLUMNS;
                                else if (h == "RHS")
                                        sec = RHS;
                                else if (h == "RANGES")
                                        sec = RANGES;
                                else if (h == "BOUNDS")
                                        sec = BOUNDS;
                                else if (h == "OBJSENSE") {
                                        sec = OBJSENSE;
                                        if (t.size() > 1)
                                                maximize = t[1] == "MAX" || t[1] == "MAXIMIZE";
                                } else if (h == "ENDATA") {
                                        sec = END;
                                        break;
                                } else {
                                        return fail("unknown section");
                                }
                                continue;
                        }
                        bool ok = true;
                        switch (sec) {
                        case ROWS: ok = row_decl(t); break;
                        case COLUMNS: ok = columns(t); break;
                        case RHS: ok = row_values(t, false); break;
                        case RANGES: ok = row_values(t, true); break;
                        case BOUNDS: ok = bound(t); break;
                        case OBJSENSE: maximize = t[0] == "MAX" || t[0] == "MAXIMIZE"; break;
                        default: ok = fail("data outside a section");
                        }
                        if (!ok)
                                return false;
                }
                if (sec != END)
                        return fail("missing ENDATA");
                return true;
        }
};

// The interval [lo, hi] of a constraint row (MPS range rules).
void row_interval(const Row & r, double & lo, double & hi)
{
        double R = std::fabs(r.range);
        switch (r.type) {
        case 'L':
                lo = r.ranged ? r.rhs - R : -HUGE_VAL;
                hi = r.rhs;
                break;
        case 'G':
                lo = r.rhs;
                hi = r.ranged ? r.rhs + R : HUGE_VAL;
                break;
        default:  // 'E'
                lo = hi = r.rhs;
                if (r.ranged) {
                        if (r.range > 0)
                                hi = r.rhs + R;
                        else
                                lo = r.rhs - R;
                }
        }
}

}  // namespace

extern "C" struct alm * acdalm_read_mps(FILE * stream)
{
        if (!stream) {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_mps: null stream");
                return nullptr;
        }
        Parser p;
        if (!p.parse(stream))
                return nullptr;
        size_t m = p.rows.size(), nx = p.col_names.size();
        std::vector<double> rhs(m, 0), lo_s, hi_s;
        std::vector<uint32_t> slack_row;
        for (size_t i = 0; i < m; i++) {
                const Row & r = p.rows[i];
                if (r.type == 'E' && !r.ranged) {
                        rhs[i] = r.rhs;
                        continue;
                }
                double lo, hi;
                row_interval(r, lo, hi);
                slack_row.push_back((uint32_t)i);
                lo_s.push_back(lo);
                hi_s.push_back(hi);
        }
        size_t n = nx + slack_row.size();
        if (m >= (1ull << 31) || n >= (1ull << 31)) {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_mps: too many rows or columns");
                return nullptr;
        }
        std::vector<uint32_t> rows, cols;
        std::vector<double> vals;
        rows.reserve(p.entries.size() + slack_row.size());
        cols.reserve(rows.capacity());
        vals.reserve(rows.capacity());
        for (const Entry & e : p.entries) {
                rows.push_back(e.row);
                cols.push_back(e.col);
                vals.push_back(e.val);
        }
        for (size_t k = 0; k < slack_row.size(); k++) {
                rows.push_back(slack_row[k]);
                cols.push_back((uint32_t)(nx + k));
                vals.push_back(-1.0);
        }
        std::vector<double> c(n, 0), l(n), u(n);
        for (size_t j = 0; j < nx; j++) {
                c[j] = p.maximize ? -p.cost[j] : p.cost[j];
                l[j] = p.lower[j];
                u[j] = p.upper[j];
        }
        for (size_t k = 0; k < slack_row.size(); k++) {
                l[nx + k] = lo_s[k];
                u[nx + k] = hi_s[k];
        }
        std::vector<double> llo(m, -HUGE_VAL), lhi(m, HUGE_VAL);
        sparse_matrix_t * mat = sparse_matrix_make(n, m, rows.size(), rows.data(), cols.data(),
                                                   vals.data(), 0);
        if (!mat)
                return nullptr;
        alm_t * out = alm_make(mat, m, rhs.data(), n, c.data(), l.data(), u.data(), llo.data(),
                               lhi.data());
        if (!out)
                sparse_matrix_free(mat);
        return out;
}

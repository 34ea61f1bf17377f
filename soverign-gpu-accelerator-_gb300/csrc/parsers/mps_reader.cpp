// Free-format MPS reader. Behaviour follows the reference's
// src/parsers/mps_reader.cpp:65-355: first N row is the objective, later N rows
// are ignored, only the first RHS / BOUNDS vector name is used, L rows get a +1
// slack and G rows a -1 surplus column (appended after the structural columns in
// row order), unknown sections / row types / bound types throw
// std::runtime_error, and a nonzero objective-row RHS throws.
#include "parsers/mps_reader.hpp"

#include <cctype>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

namespace sankhya {
namespace parsers {

namespace {

struct RowRec {
    char kind;
    Float rhs = 0.0;
    bool has_rhs = false;
    std::vector<Index> cols;
    std::vector<Float> vals;
    Index slack = -1;
};

struct ColRec {
    Float cost = 0.0;
    Float lo = 0.0;
    Float hi = math::kInfinity;
    VariableType vt = VariableType::Continuous;
};

std::vector<std::string> tokens_of(const std::string& s) {
    std::vector<std::string> out;
    std::istringstream is(s);
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
}

Float number(const std::string& tok, const char* where, int line) {
    try {
        size_t used = 0;
        Float v = std::stod(tok, &used);
        if (used != tok.size()) throw std::invalid_argument(tok);
        return v;
    } catch (...) {
        throw std::runtime_error(std::string("MPS parser error: Invalid numeric value in ") + where +
                                 " at line " + std::to_string(line));
    }
}

}  // namespace

core::Model read_mps(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.is_open()) throw std::runtime_error("MPS parser error: Could not open file " + filename);

    enum class Sec { None, Name, Rows, Columns, Rhs, Bounds } sec = Sec::None;
    std::vector<RowRec> rows;
    std::unordered_map<std::string, Index> row_id;
    Index objective_row = -1;
    std::vector<ColRec> cols;
    std::unordered_map<std::string, Index> col_id;
    bool integer_block = false;
    std::string rhs_set, bound_set;
    std::string line;
    int lineno = 0;

    while (std::getline(in, line)) {
        ++lineno;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty() || line[0] == '*') continue;
        auto tok = tokens_of(line);
        if (tok.empty()) continue;
        if (!std::isspace(static_cast<unsigned char>(line[0]))) {
            const std::string& h = tok[0];
            if (h == "NAME") sec = Sec::Name;
            else if (h == "ROWS") sec = Sec::Rows;
            else if (h == "COLUMNS") sec = Sec::Columns;
            else if (h == "RHS") sec = Sec::Rhs;
            else if (h == "BOUNDS") sec = Sec::Bounds;
            else if (h == "ENDATA") break;
            else
                throw std::runtime_error("MPS parser error: Unsupported section '" + h + "' at line " +
                                         std::to_string(lineno));
            continue;
        }
        switch (sec) {
        case Sec::Rows: {
            if (tok.size() < 2)
                throw std::runtime_error("MPS parser error: Malformed ROWS record at line " + std::to_string(lineno));
            const char k = tok[0][0];
            if (k != 'N' && k != 'L' && k != 'G' && k != 'E')
                throw std::runtime_error(std::string("MPS parser error: Unknown row type '") + k + "' at line " +
                                         std::to_string(lineno));
            if (k == 'N' && objective_row < 0) objective_row = static_cast<Index>(rows.size());
            row_id[tok[1]] = static_cast<Index>(rows.size());
            RowRec r;
            r.kind = k;
            rows.push_back(std::move(r));
            break;
        }
        case Sec::Columns: {
            if (tok.size() < 3)
                throw std::runtime_error("MPS parser error: Malformed COLUMNS record at line " + std::to_string(lineno));
            if (tok[1] == "'MARKER'") {
                if (tok[2] == "'INTORG'") integer_block = true;
                else if (tok[2] == "'INTEND'") integer_block = false;
                break;
            }
            auto it = col_id.find(tok[0]);
            Index j;
            if (it == col_id.end()) {
                j = static_cast<Index>(cols.size());
                col_id.emplace(tok[0], j);
                ColRec c;
                c.vt = integer_block ? VariableType::Integer : VariableType::Continuous;
                cols.push_back(c);
            } else {
                j = it->second;
            }
            for (size_t t = 1; t < tok.size(); t += 2) {
                if (t + 1 >= tok.size())
                    throw std::runtime_error("MPS parser error: Missing value for row in COLUMNS at line " +
                                             std::to_string(lineno));
                const Float v = number(tok[t + 1], "COLUMNS", lineno);
                auto r = row_id.find(tok[t]);
                if (r == row_id.end())
                    throw std::runtime_error("MPS parser error: Reference to unknown row '" + tok[t] + "' in COLUMNS");
                if (r->second == objective_row) {
                    cols[static_cast<size_t>(j)].cost = v;
                } else {
                    rows[static_cast<size_t>(r->second)].cols.push_back(j);
                    rows[static_cast<size_t>(r->second)].vals.push_back(v);
                }
            }
            break;
        }
        case Sec::Rhs: {
            if (tok.size() < 3)
                throw std::runtime_error("MPS parser error: Malformed RHS record at line " + std::to_string(lineno));
            if (rhs_set.empty()) rhs_set = tok[0];
            else if (tok[0] != rhs_set) break;
            for (size_t t = 1; t < tok.size(); t += 2) {
                if (t + 1 >= tok.size())
                    throw std::runtime_error("MPS parser error: Missing value for row in RHS at line " +
                                             std::to_string(lineno));
                const Float v = number(tok[t + 1], "RHS", lineno);
                auto r = row_id.find(tok[t]);
                if (r == row_id.end())
                    throw std::runtime_error("MPS parser error: Reference to unknown row '" + tok[t] + "' in RHS");
                rows[static_cast<size_t>(r->second)].rhs = v;
                rows[static_cast<size_t>(r->second)].has_rhs = true;
            }
            break;
        }
        case Sec::Bounds: {
            if (tok.size() < 3)
                throw std::runtime_error("MPS parser error: Malformed BOUNDS record at line " + std::to_string(lineno));
            if (bound_set.empty()) bound_set = tok[1];
            else if (tok[1] != bound_set) break;
            auto c = col_id.find(tok[2]);
            if (c == col_id.end())
                throw std::runtime_error("MPS parser error: Reference to unknown column '" + tok[2] + "' in BOUNDS");
            ColRec& col = cols[static_cast<size_t>(c->second)];
            const std::string& bt = tok[0];
            auto value = [&]() {
                if (tok.size() < 4) throw std::runtime_error("MPS parser error: " + bt + " bound missing value");
                return number(tok[3], "BOUNDS", lineno);
            };
            if (bt == "LO") col.lo = value();
            else if (bt == "UP") col.hi = value();
            else if (bt == "FX") col.lo = col.hi = value();
            else if (bt == "FR") { col.lo = -math::kInfinity; col.hi = math::kInfinity; }
            else if (bt == "MI") col.lo = -math::kInfinity;
            else if (bt == "PL") col.hi = math::kInfinity;
            else if (bt == "BV") { col.vt = VariableType::Binary; col.lo = 0.0; col.hi = 1.0; }
            else if (bt == "LI") { col.vt = VariableType::Integer; col.lo = value(); }
            else if (bt == "UI") { col.vt = VariableType::Integer; col.hi = value(); }
            else throw std::runtime_error("MPS parser error: Unsupported bound type '" + bt + "'");
            break;
        }
        default:
            break;
        }
    }

    core::Model model;
    for (const auto& c : cols) model.add_variable(c.cost, c.lo, c.hi, c.vt);
    Index next = static_cast<Index>(cols.size());
    for (auto& r : rows) {
        if (r.kind == 'L' || r.kind == 'G') {
            r.slack = next++;
            model.add_variable(0.0, 0.0, math::kInfinity, VariableType::Continuous);
        }
    }
    for (const auto& r : rows) {
        if (r.kind == 'N') {
            if (r.has_rhs && r.rhs != 0.0)
                throw std::runtime_error(
                    "MPS parser error: Objective row RHS (constant offset) is not supported by the current Model API.");
            continue;
        }
        std::vector<Index> cc = r.cols;
        std::vector<Float> vv = r.vals;
        if (r.slack >= 0) {
            cc.push_back(r.slack);
            vv.push_back(r.kind == 'L' ? 1.0 : -1.0);
        }
        model.add_constraint(cc, vv, r.rhs);
    }
    model.sense = OptimizationSense::Minimize;
    model.finalize();
    return model;
}

}  // namespace parsers
}  // namespace sankhya

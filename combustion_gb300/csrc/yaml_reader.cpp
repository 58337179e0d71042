// Cantera-YAML mechanism reader: the subset that the reference's loader reads (yaml.rs:54-171) and the
// species arrays its builder derives (lib.rs:20-54, Reaction::new lib.rs:100-125), filling a cb_mech_desc.
//
// The YAML side is a small parser of its own: block mappings and sequences by indentation, flow
// collections ([...], {...}, possibly over several lines), plain and quoted scalars, comments, and block
// scalars (|, >) kept as text. That covers Cantera's mechanism files; anchors, tags and multi-document
// streams are not supported.
//
// Model semantics follow the reference: units must be cm, s and mol with the activation energy in K or
// cal/mol; A is converted by 1e-6^(order - 1) (three-body reactions count M in the order, a falloff k0 by
// 1e-6^order); molar masses from the composition with the standard atomic weights of lib.rs:21-23; NASA-7
// pieces split at the middle temperature, or one piece when two equal pieces were written (the
// duplicate-spline merge of yaml.rs:64-77); well depth K -> J, diameter A -> m, polarizability A^3 -> m^3
// (linear and nonlinear molecules), dipole Debye -> C m (nonlinear only), rotational relaxation as given;
// reaction types elementary / irreversible ("=>"), three-body, falloff (Troe, SRI or Lindemann) and
// pressure-dependent-Arrhenius with one rate; efficiencies default to 1; species reordered with the
// species some reaction changes first, each group in file order (yaml.rs:159-162).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"
#include "capi_internal.h"

namespace {

struct YNode {
    enum Kind { Null, Scalar, Seq, Map } kind = Null;
    std::string text;
    std::vector<YNode> items;
    std::vector<std::pair<std::string, YNode>> entries;
    const YNode* get(const std::string& k) const {
        if (kind != Map) return nullptr;
        for (const auto& e : entries)
            if (e.first == k) return &e.second;
        return nullptr;
    }
};

struct ParseError {
    std::string msg;
};

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r')) a++;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) b--;
    return s.substr(a, b - a);
}

// Position of a comment '#' (outside quotes, at the start or after whitespace), or npos.
size_t comment_pos(const std::string& s) {
    char q = 0;
    for (size_t i = 0; i < s.size(); i++) {
        const char c = s[i];
        if (q) {
            if (c == q) q = 0;
        } else if (c == '\'' || c == '"') {
            q = c;
        } else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) {
            return i;
        }
    }
    return std::string::npos;
}

struct Line {
    int indent;
    std::string text;
};

class Parser {
   public:
    explicit Parser(const std::string& src) {
        size_t start = 0;
        while (start <= src.size()) {
            size_t end = src.find('\n', start);
            if (end == std::string::npos) end = src.size();
            raw_.push_back(src.substr(start, end - start));
            start = end + 1;
        }
    }
    YNode parse() {
        build_lines();
        size_t i = 0;
        if (lines_.empty()) return YNode();
        return block(i, lines_[0].indent);
    }

   private:
    std::vector<std::string> raw_;
    std::vector<Line> lines_;
    std::vector<size_t> raw_index_;  // raw line of each logical line (block scalars)

    void build_lines() {
        for (size_t r = 0; r < raw_.size(); r++) {
            std::string s = raw_[r];
            if (!s.empty() && s.back() == '\r') s.pop_back();
            int ind = 0;
            while (ind < (int)s.size() && s[ind] == ' ') ind++;
            std::string body = s.substr(ind);
            if (body.rfind("---", 0) == 0 || body.rfind("...", 0) == 0) continue;
            const size_t c = comment_pos(body);
            if (c != std::string::npos) body = body.substr(0, c);
            body = trim(body);
            if (body.empty()) continue;
            if (body[0] == '\t') throw ParseError{"tab indentation"};
            lines_.push_back({ind, body});
            raw_index_.push_back(r);
        }
    }

    static bool is_seq_item(const std::string& t) { return t == "-" || t.rfind("- ", 0) == 0; }

    // Splits "key: value" at the first ':' followed by a space or the end (outside quotes and brackets).
    static bool split_key(const std::string& t, std::string& key, std::string& rest) {
        char q = 0;
        int depth = 0;
        for (size_t i = 0; i < t.size(); i++) {
            const char c = t[i];
            if (q) {
                if (c == q) q = 0;
                continue;
            }
            if (c == '\'' || c == '"') q = c;
            else if (c == '[' || c == '{') depth++;
            else if (c == ']' || c == '}') depth--;
            else if (c == ':' && depth == 0 && (i + 1 == t.size() || t[i + 1] == ' ')) {
                key = unquote(trim(t.substr(0, i)));
                rest = trim(t.substr(i + 1));
                return true;
            }
        }
        return false;
    }

    static std::string unquote(const std::string& s) {
        if (s.size() >= 2 && ((s.front() == '\'' && s.back() == '\'') || (s.front() == '"' && s.back() == '"')))
            return s.substr(1, s.size() - 2);
        return s;
    }

    static bool balanced(const std::string& s) {
        int depth = 0;
        char q = 0;
        for (char c : s) {
            if (q) {
                if (c == q) q = 0;
                continue;
            }
            if (c == '\'' || c == '"') q = c;
            else if (c == '[' || c == '{') depth++;
            else if (c == ']' || c == '}') depth--;
        }
        return depth <= 0;
    }

    // Value text that starts on line i (already split off): flow collections may continue on later lines.
    YNode value(const std::string& first, size_t& i, int indent) {
        if (first.empty()) {  // nested block (deeper, or a sequence at the key's own indent)
            if (i < lines_.size() && (lines_[i].indent > indent || (lines_[i].indent == indent && is_seq_item(lines_[i].text))))
                return block(i, lines_[i].indent);
            return YNode();
        }
        if (first[0] == '|' || first[0] == '>') {  // block scalar: lines indented deeper than the key
            YNode n;
            n.kind = YNode::Scalar;
            while (i < lines_.size() && lines_[i].indent > indent) n.text += lines_[i++].text + "\n";
            return n;
        }
        if (first[0] == '[' || first[0] == '{') {
            std::string s = first;
            while (!balanced(s) && i < lines_.size()) s += " " + lines_[i++].text;
            size_t pos = 0;
            return flow(s, pos);
        }
        YNode n;
        n.kind = YNode::Scalar;
        n.text = unquote(first);
        return n;
    }

    YNode block(size_t& i, int indent) {
        YNode node;
        if (i >= lines_.size()) return node;
        if (is_seq_item(lines_[i].text)) {
            node.kind = YNode::Seq;
            while (i < lines_.size() && lines_[i].indent == indent && is_seq_item(lines_[i].text)) {
                std::string t = lines_[i].text == "-" ? "" : trim(lines_[i].text.substr(2));
                i++;
                if (t.empty()) {
                    node.items.push_back(value("", i, indent));
                    continue;
                }
                std::string key, rest;
                if (t[0] != '[' && t[0] != '{' && t[0] != '\'' && t[0] != '"' && split_key(t, key, rest)) {
                    // "- key: value" opens a mapping whose other entries sit at the key's column
                    const int col = indent + 2 + (int)(lines_[i - 1].text.size() - 2 - trim(lines_[i - 1].text.substr(2)).size());
                    YNode m;
                    m.kind = YNode::Map;
                    m.entries.emplace_back(key, value(rest, i, col));
                    while (i < lines_.size() && lines_[i].indent == col && !is_seq_item(lines_[i].text)) {
                        std::string k2, r2;
                        if (!split_key(lines_[i].text, k2, r2)) throw ParseError{"expected 'key: value': " + lines_[i].text};
                        i++;
                        m.entries.emplace_back(k2, value(r2, i, col));
                    }
                    node.items.push_back(std::move(m));
                } else {
                    node.items.push_back(value(t, i, indent));
                }
            }
            return node;
        }
        node.kind = YNode::Map;
        while (i < lines_.size() && lines_[i].indent == indent && !is_seq_item(lines_[i].text)) {
            std::string key, rest;
            if (!split_key(lines_[i].text, key, rest)) throw ParseError{"expected 'key: value': " + lines_[i].text};
            i++;
            node.entries.emplace_back(key, value(rest, i, indent));
        }
        return node;
    }

    static void skip_ws(const std::string& s, size_t& p) {
        while (p < s.size() && (s[p] == ' ' || s[p] == '\t')) p++;
    }

    static YNode flow(const std::string& s, size_t& p) {
        skip_ws(s, p);
        YNode n;
        if (p >= s.size()) return n;
        if (s[p] == '[') {
            n.kind = YNode::Seq;
            p++;
            for (;;) {
                skip_ws(s, p);
                if (p >= s.size()) throw ParseError{"unterminated '['"};
                if (s[p] == ']') {
                    p++;
                    break;
                }
                n.items.push_back(flow(s, p));
                skip_ws(s, p);
                if (p < s.size() && s[p] == ',') p++;
            }
            return n;
        }
        if (s[p] == '{') {
            n.kind = YNode::Map;
            p++;
            for (;;) {
                skip_ws(s, p);
                if (p >= s.size()) throw ParseError{"unterminated '{'"};
                if (s[p] == '}') {
                    p++;
                    break;
                }
                std::string key = scalar_text(s, p, true);
                skip_ws(s, p);
                if (p >= s.size() || s[p] != ':') throw ParseError{"expected ':' in a flow mapping"};
                p++;
                n.entries.emplace_back(key, flow(s, p));
                skip_ws(s, p);
                if (p < s.size() && s[p] == ',') p++;
            }
            return n;
        }
        n.kind = YNode::Scalar;
        n.text = scalar_text(s, p, false);
        return n;
    }

    static std::string scalar_text(const std::string& s, size_t& p, bool key) {
        skip_ws(s, p);
        if (p < s.size() && (s[p] == '\'' || s[p] == '"')) {
            const char q = s[p++];
            size_t e = s.find(q, p);
            if (e == std::string::npos) throw ParseError{"unterminated quote"};
            std::string t = s.substr(p, e - p);
            p = e + 1;
            return t;
        }
        size_t b = p;
        while (p < s.size() && s[p] != ',' && s[p] != ']' && s[p] != '}' && !(key && s[p] == ':')) p++;
        return trim(s.substr(b, p - b));
    }
};

bool number(const YNode* n, double& v) {
    if (!n || n->kind != YNode::Scalar) return false;
    const std::string& t = n->text;
    if (t == ".inf" || t == ".Inf" || t == "inf") {
        v = INFINITY;
        return true;
    }
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == 0 && !t.empty();
}

constexpr double kB = 1.380649e-23, NA = 6.02214076e23, R = kB * NA;
constexpr double kJPerCal = 4.184;
constexpr double kCmPerDebye = 1e-21 / 299792458.0;

double atomic_weight(const std::string& e, bool& ok) {  // kg/mol (lib.rs:21-23)
    static const std::map<std::string, double> w = {{"H", 1.008},   {"He", 4.002602}, {"C", 12.011},
                                                    {"N", 14.007},  {"O", 15.999},    {"F", 18.998403163},
                                                    {"Cl", 35.45}, {"Ar", 39.95}};
    auto it = w.find(e);
    ok = it != w.end();
    return ok ? it->second / 1e3 : 0.0;
}

struct Equation {
    std::vector<std::pair<std::string, int>> sides[2];
    bool reversible = true;
};

std::string trim_suffix(std::string s, const std::string& suf) {
    while (s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0) s.erase(s.size() - suf.size());
    return s;
}

// yaml.rs equation(): split at "<=>" or "=>", drop a trailing "(+ M)" / "+ M" / "(+M)", terms separated by
// " + ", "count species" or "species".
bool parse_equation(const std::string& eq, Equation& out, std::string& err) {
    std::string a, b;
    size_t p = eq.find("<=>");
    if (p != std::string::npos) {
        a = eq.substr(0, p);
        b = eq.substr(p + 3);
        out.reversible = true;
    } else if ((p = eq.find("=>")) != std::string::npos) {
        a = eq.substr(0, p);
        b = eq.substr(p + 2);
        out.reversible = false;
    } else {
        err = "equation without '<=>' or '=>': " + eq;
        return false;
    }
    const std::string sides[2] = {a, b};
    for (int s = 0; s < 2; s++) {
        std::string t = trim(sides[s]);
        t = trim_suffix(t, "(+ M)");
        t = trim_suffix(t, "+ M");
        t = trim_suffix(t, "(+M)");
        size_t start = 0;
        for (;;) {
            size_t q = t.find(" + ", start);
            std::string term = trim(t.substr(start, q == std::string::npos ? std::string::npos : q - start));
            if (!term.empty()) {
                int count = 1;
                std::string name = term;
                const size_t sp = term.find_first_of(" \t");
                if (sp != std::string::npos) {
                    const std::string c = trim(term.substr(0, sp));
                    name = trim(term.substr(sp + 1));
                    char* end = nullptr;
                    count = (int)std::strtol(c.c_str(), &end, 10);
                    if (!end || *end != 0 || count <= 0) {
                        err = "bad stoichiometric term '" + term + "' in " + eq;
                        return false;
                    }
                }
                bool merged = false;
                for (auto& e : out.sides[s])
                    if (e.first == name) {
                        e.second += count;
                        merged = true;
                    }
                if (!merged) out.sides[s].emplace_back(name, count);
            }
            if (q == std::string::npos) break;
            start = q + 3;
        }
    }
    return true;
}

}  // namespace

struct cb_yaml_mech {
    std::vector<std::string> names;
    std::vector<double> molar_mass, split, nasa7, diameter, well_depth, polarizability, dipole, rot;
    std::vector<int32_t> geometry, model;
    std::vector<uint8_t> reactants, products;
    std::vector<double> rate, k0, troe, sri, eff;
    int K = 0, R = 0;
};

namespace {

int build(const YNode& root, cb_yaml_mech& m, std::string& err) {
    const YNode* units = root.get("units");
    auto unit = [&](const char* k) -> std::string {
        const YNode* u = units ? units->get(k) : nullptr;
        return u && u->kind == YNode::Scalar ? u->text : std::string();
    };
    if (unit("length") != "cm" || unit("time") != "s" || unit("quantity") != "mol") {
        err = "units must be length: cm, time: s, quantity: mol (yaml.rs:57)";
        return CB_ERR_MECHANISM;
    }
    const std::string ea_unit = unit("activation-energy");
    if (ea_unit != "K" && ea_unit != "cal/mol") {
        err = "activation-energy unit must be K or cal/mol";
        return CB_ERR_MECHANISM;
    }
    const YNode* species = root.get("species");
    const YNode* reactions = root.get("reactions");
    if (!species || species->kind != YNode::Seq || !reactions || reactions->kind != YNode::Seq) {
        err = "missing species or reactions";
        return CB_ERR_MECHANISM;
    }
    struct Sp {
        std::string name;
        double W = 0, split = NAN, nasa[2][7] = {}, diameter = 0, well = 0, polar = 0, dipole = 0, rot = 0;
        int geometry = 0;
    };
    std::vector<Sp> sp;
    for (const YNode& s : species->items) {
        Sp x;
        const YNode* name = s.get("name");
        if (!name || name->kind != YNode::Scalar) {
            err = "species without a name";
            return CB_ERR_MECHANISM;
        }
        x.name = name->text;
        const YNode* comp = s.get("composition");
        if (!comp || comp->kind != YNode::Map) {
            err = x.name + ": no composition";
            return CB_ERR_MECHANISM;
        }
        for (const auto& e : comp->entries) {
            double c;
            bool ok;
            const double w = atomic_weight(e.first, ok);
            if (!ok || !number(&e.second, c)) {
                err = x.name + ": element " + e.first + " outside H He C N O F Cl Ar";
                return CB_ERR_MECHANISM;
            }
            x.W += c * w;
        }
        const YNode* thermo = s.get("thermo");
        const YNode* ranges = thermo ? thermo->get("temperature-ranges") : nullptr;
        const YNode* data = thermo ? thermo->get("data") : nullptr;
        if (!ranges || ranges->kind != YNode::Seq || !data || data->kind != YNode::Seq || data->items.empty() ||
            data->items.size() > 2 || ranges->items.size() != data->items.size() + 1) {
            err = x.name + ": thermo needs NASA-7 data with 1 or 2 pieces";
            return CB_ERR_MECHANISM;
        }
        double pieces[2][7];
        for (size_t q = 0; q < data->items.size(); q++) {
            const YNode& piece = data->items[q];
            if (piece.kind != YNode::Seq || piece.items.size() != 7) {
                err = x.name + ": NASA-7 piece without 7 coefficients";
                return CB_ERR_MECHANISM;
            }
            for (int j = 0; j < 7; j++)
                if (!number(&piece.items[j], pieces[q][j])) {
                    err = x.name + ": bad NASA-7 coefficient";
                    return CB_ERR_MECHANISM;
                }
        }
        bool one = data->items.size() == 1;
        if (!one) {  // duplicate splines (yaml.rs:64-77): equal a0..a5 and a6 within 3e-8
            bool same = std::fabs(pieces[0][6] - pieces[1][6]) < 3e-8;
            for (int j = 0; j < 6; j++) same &= pieces[0][j] == pieces[1][j];
            one = same;
        }
        if (one) {
            x.split = NAN;
            for (int j = 0; j < 7; j++) x.nasa[0][j] = x.nasa[1][j] = pieces[0][j];
        } else {
            if (!number(&ranges->items[1], x.split)) {
                err = x.name + ": bad temperature range";
                return CB_ERR_MECHANISM;
            }
            for (int q = 0; q < 2; q++)
                for (int j = 0; j < 7; j++) x.nasa[q][j] = pieces[q][j];
        }
        const YNode* tr = s.get("transport");
        double v;
        if (!tr || !number(tr->get("well-depth"), v)) {
            err = x.name + ": transport data needed (well-depth, diameter, geometry)";
            return CB_ERR_MECHANISM;
        }
        x.well = v * kB;
        if (!number(tr->get("diameter"), v)) {
            err = x.name + ": no diameter";
            return CB_ERR_MECHANISM;
        }
        x.diameter = v * 1e-10;
        const YNode* geo = tr->get("geometry");
        const std::string g = geo && geo->kind == YNode::Scalar ? geo->text : "";
        if (g == "atom") x.geometry = CB_ATOM;
        else if (g == "linear") x.geometry = CB_LINEAR;
        else if (g == "nonlinear") x.geometry = CB_NONLINEAR;
        else {
            err = x.name + ": geometry must be atom, linear or nonlinear";
            return CB_ERR_MECHANISM;
        }
        if (x.geometry != CB_ATOM) {
            if (number(tr->get("polarizability"), v)) x.polar = v * 1e-30;
            if (number(tr->get("rotational-relaxation"), v)) x.rot = v;
        }
        if (x.geometry == CB_NONLINEAR && number(tr->get("dipole"), v)) x.dipole = v * kCmPerDebye;
        sp.push_back(x);
    }
    const int K = (int)sp.size();
    std::map<std::string, int> index;
    for (int k = 0; k < K; k++) index[sp[k].name] = k;
    struct Rx {
        std::vector<int> lhs, rhs;
        int model = 0;
        double rate[3] = {}, k0[3] = {}, troe[4] = {}, sri[5] = {};
        std::vector<double> eff;
    };
    std::vector<Rx> rx;
    auto rate_constant = [&](const YNode* rc, int exponent, double out[3]) -> bool {
        double A, b, Ea;
        if (!rc || !number(rc->get("A"), A) || !number(rc->get("b"), b) || !number(rc->get("Ea"), Ea)) return false;
        out[0] = A * std::pow(1e-6, (double)exponent);
        out[1] = b;
        out[2] = ea_unit == "K" ? Ea : Ea * kJPerCal / R;
        return true;
    };
    for (const YNode& r : reactions->items) {
        const YNode* eqn = r.get("equation");
        Equation eq;
        if (!eqn || eqn->kind != YNode::Scalar || !parse_equation(eqn->text, eq, err)) {
            if (err.empty()) err = "reaction without an equation";
            return CB_ERR_MECHANISM;
        }
        Rx x;
        x.lhs.assign(K, 0);
        x.rhs.assign(K, 0);
        for (int s = 0; s < 2; s++)
            for (const auto& t : eq.sides[s]) {
                auto it = index.find(t.first);
                if (it == index.end()) {
                    err = "unknown species '" + t.first + "' in " + eqn->text;
                    return CB_ERR_MECHANISM;
                }
                (s ? x.rhs : x.lhs)[it->second] += t.second;
            }
        const YNode* type = r.get("type");
        const std::string ty = type && type->kind == YNode::Scalar ? type->text : "elementary";
        int reactants = 0;
        for (int c : x.lhs) reactants += c;
        if (ty == "three-body") reactants += 1;
        const YNode* rc = r.get("rate-constant");
        if (!rc) rc = r.get("high-P-rate-constant");
        if (!rc) {
            const YNode* list = r.get("rate-constants");
            if (ty != "pressure-dependent-Arrhenius" || !list || list->kind != YNode::Seq || list->items.size() != 1) {
                err = eqn->text + ": pressure-dependent-Arrhenius rates need exactly one rate (yaml.rs:148-153)";
                return CB_ERR_UNSUPPORTED;
            }
            rc = &list->items[0];
        }
        if (!rate_constant(rc, reactants - 1, x.rate)) {
            err = eqn->text + ": bad rate constant";
            return CB_ERR_MECHANISM;
        }
        x.eff.assign(K, 1.0);
        if (const YNode* e = r.get("efficiencies")) {
            if (e->kind != YNode::Map) {
                err = eqn->text + ": efficiencies must be a mapping";
                return CB_ERR_MECHANISM;
            }
            for (const auto& kv : e->entries) {
                auto it = index.find(kv.first);
                double v;
                if (it == index.end() || !number(&kv.second, v)) {
                    err = eqn->text + ": bad efficiency for " + kv.first;
                    return CB_ERR_MECHANISM;
                }
                x.eff[it->second] = v;
            }
        }
        if (ty == "elementary" || ty == "pressure-dependent-Arrhenius") {
            x.model = eq.reversible ? CB_ELEMENTARY : CB_IRREVERSIBLE;
        } else if (ty == "three-body") {
            x.model = CB_THREE_BODY;
        } else if (ty == "falloff") {
            if (!rate_constant(r.get("low-P-rate-constant"), reactants, x.k0)) {
                err = eqn->text + ": falloff without low-P-rate-constant";
                return CB_ERR_MECHANISM;
            }
            if (const YNode* t = r.get("Troe")) {
                x.model = CB_TROE;
                if (!number(t->get("A"), x.troe[0]) || !number(t->get("T3"), x.troe[1]) || !number(t->get("T1"), x.troe[2])) {
                    err = eqn->text + ": Troe needs A, T3, T1";
                    return CB_ERR_MECHANISM;
                }
                if (!number(t->get("T2"), x.troe[3])) x.troe[3] = INFINITY;
            } else if (const YNode* s = r.get("SRI")) {
                x.model = CB_SRI;
                if (!number(s->get("A"), x.sri[0]) || !number(s->get("B"), x.sri[1]) || !number(s->get("C"), x.sri[2])) {
                    err = eqn->text + ": SRI needs A, B, C";
                    return CB_ERR_MECHANISM;
                }
                if (!number(s->get("D"), x.sri[3])) x.sri[3] = 1.0;
                if (!number(s->get("E"), x.sri[4])) x.sri[4] = 0.0;
            } else {
                x.model = CB_LINDEMANN;
            }
        } else {
            err = eqn->text + ": reaction type '" + ty + "' is not read (yaml.rs:124-155)";
            return CB_ERR_UNSUPPORTED;
        }
        rx.push_back(std::move(x));
    }
    // active species first, each group in file order (yaml.rs:159-162)
    std::vector<int> order;
    std::vector<char> changes(K, 0);
    for (const Rx& x : rx)
        for (int k = 0; k < K; k++) changes[k] |= x.lhs[k] != x.rhs[k];
    for (int k = 0; k < K; k++)
        if (changes[k]) order.push_back(k);
    for (int k = 0; k < K; k++)
        if (!changes[k]) order.push_back(k);
    const int R_ = (int)rx.size();
    m.K = K;
    m.R = R_;
    m.names.resize(K);
    m.molar_mass.resize(K);
    m.split.resize(K);
    m.nasa7.resize((size_t)K * 14);
    m.geometry.resize(K);
    m.diameter.resize(K);
    m.well_depth.resize(K);
    m.polarizability.resize(K);
    m.dipole.resize(K);
    m.rot.resize(K);
    for (int i = 0; i < K; i++) {
        const Sp& x = sp[order[i]];
        m.names[i] = x.name;
        m.molar_mass[i] = x.W;
        m.split[i] = x.split;
        for (int q = 0; q < 2; q++)
            for (int j = 0; j < 7; j++) m.nasa7[(size_t)i * 14 + q * 7 + j] = x.nasa[q][j];
        m.geometry[i] = x.geometry;
        m.diameter[i] = x.diameter;
        m.well_depth[i] = x.well;
        m.polarizability[i] = x.polar;
        m.dipole[i] = x.dipole;
        m.rot[i] = x.rot;
    }
    m.reactants.assign((size_t)R_ * K, 0);
    m.products.assign((size_t)R_ * K, 0);
    m.model.resize(R_);
    m.rate.resize((size_t)R_ * 3);
    m.k0.assign((size_t)R_ * 3, 0.0);
    m.troe.assign((size_t)R_ * 4, 0.0);
    m.sri.assign((size_t)R_ * 5, 0.0);
    m.eff.assign((size_t)R_ * K, 1.0);
    for (int r = 0; r < R_; r++) {
        const Rx& x = rx[r];
        for (int i = 0; i < K; i++) {
            const int k = order[i];
            if (x.lhs[k] > 255 || x.rhs[k] > 255) {
                err = "stoichiometric coefficient above 255";
                return CB_ERR_MECHANISM;
            }
            m.reactants[(size_t)r * K + i] = (uint8_t)x.lhs[k];
            m.products[(size_t)r * K + i] = (uint8_t)x.rhs[k];
            m.eff[(size_t)r * K + i] = x.eff[k];
        }
        m.model[r] = x.model;
        for (int j = 0; j < 3; j++) {
            m.rate[(size_t)r * 3 + j] = x.rate[j];
            m.k0[(size_t)r * 3 + j] = x.k0[j];
        }
        for (int j = 0; j < 4; j++) m.troe[(size_t)r * 4 + j] = x.troe[j];
        for (int j = 0; j < 5; j++) m.sri[(size_t)r * 5 + j] = x.sri[j];
    }
    return CB_OK;
}

}  // namespace

extern "C" {

int cb_yaml_load(const char* text, size_t len, cb_yaml_mech** out) {
    if (!text || !out) return cbi::fail(CB_ERR_INVALID, "null argument");
    *out = nullptr;
    YNode root;
    try {
        Parser p(std::string(text, len));
        root = p.parse();
    } catch (const ParseError& e) {
        return cbi::fail(CB_ERR_MECHANISM, "YAML: " + e.msg);
    }
    if (root.kind != YNode::Map) return cbi::fail(CB_ERR_MECHANISM, "YAML: the document is not a mapping");
    auto m = std::make_unique<cb_yaml_mech>();
    std::string err;
    const int rc = build(root, *m, err);
    if (rc) return cbi::fail(rc, err);
    *out = m.release();
    return CB_OK;
}

int cb_yaml_desc(const cb_yaml_mech* m, cb_mech_desc* d) {
    if (!m || !d) return cbi::fail(CB_ERR_INVALID, "null argument");
    d->n_species = m->K;
    d->n_reactions = m->R;
    d->molar_mass = m->molar_mass.data();
    d->nasa7_split = m->split.data();
    d->nasa7 = m->nasa7.data();
    d->geometry = m->geometry.data();
    d->diameter = m->diameter.data();
    d->well_depth = m->well_depth.data();
    d->polarizability = m->polarizability.data();
    d->dipole = m->dipole.data();
    d->rotational_relaxation = m->rot.data();
    d->reactants = m->reactants.data();
    d->products = m->products.data();
    d->model = m->model.data();
    d->rate = m->rate.data();
    d->k0 = m->k0.data();
    d->troe = m->troe.data();
    d->sri = m->sri.data();
    d->efficiencies = m->eff.data();
    return CB_OK;
}

const char* cb_yaml_species_name(const cb_yaml_mech* m, int32_t k) {
    if (!m || k < 0 || k >= m->K) return nullptr;
    return m->names[k].c_str();
}

int cb_yaml_free(cb_yaml_mech* m) {
    delete m;
    return CB_OK;
}

}  // extern "C"

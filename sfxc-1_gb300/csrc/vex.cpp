// VEX parser and queries; see vex.hpp.  The token rules restate the flex
// scanner (sfxc/lib/vex_parser/vex_parser/src/vex_scanner.ll), the grammar
// the bison one (vex_parser.yy:20-160), the unit table and date arithmetic
// Vexpp_node.cc:174-260,390-480, the queries Vex++.cc:36-239.
#include "vex.hpp"

#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace sfxc {

// ---------------------------------------------------------------- tree

const VexNode *VexNode::get(const std::string &key) const {
  if (kind != DICT) throw std::runtime_error("vex: '" + key + "' looked up in a value that is not a block");
  auto it = dict.lower_bound(key);
  if (it == dict.end() || it->first != key) return nullptr;
  return &it->second;
}

std::vector<const VexNode *> VexNode::all(const std::string &key) const {
  std::vector<const VexNode *> out;
  if (kind != DICT) return out;
  auto r = dict.equal_range(key);
  for (auto it = r.first; it != r.second; ++it) out.push_back(&it->second);
  return out;
}

const VexNode &VexNode::at(size_t i) const {
  if (kind != LIST || i >= list.size())
    throw std::runtime_error("vex: field " + std::to_string(i) + " of a statement that has no such field" +
                             (kind == STR ? " ('" + s + "')" : std::string()));
  return list[i];
}

const std::string &VexNode::str() const {
  if (kind != STR) throw std::runtime_error("vex: a list or block where a single value is expected");
  return s;
}

int VexNode::to_int() const {
  int v;
  if (std::sscanf(str().c_str(), "%d", &v) != 1) throw std::runtime_error("vex: not an integer: '" + s + "'");
  return v;
}

double VexNode::to_double() const {
  double v;
  if (std::sscanf(str().c_str(), "%lf", &v) != 1) throw std::runtime_error("vex: not a number: '" + s + "'");
  return v;
}

namespace {

// Single units: dimension and scale to the SI unit (Vexpp_node.cc:174-246).
bool unit_info(const std::string &u, std::string &dim, double &scale) {
  static const struct {
    const char *name, *dim;
    double scale;
  } table[] = {
      {"um", "length", 1e-6},  {"mm", "length", 1e-3},   {"cm", "length", 1e-2},   {"m", "length", 1},
      {"km", "length", 1e3},   {"psec", "time", 1e-12},  {"nsec", "time", 1e-9},   {"usec", "time", 1e-6},
      {"msec", "time", 1e-3},  {"sec", "time", 1},       {"min", "time", 60},      {"hr", "time", 3600},
      {"yr", "time", 365.25 * 86400},                    {"mHz", "frequency", 1e-3}, {"Hz", "frequency", 1},
      {"kHz", "frequency", 1e3}, {"MHz", "frequency", 1e6}, {"GHz", "frequency", 1e9},
  };
  for (const auto &t : table)
    if (u == t.name) {
      dim = t.dim;
      scale = t.scale;
      return true;
    }
  // a ratio: length/time is a velocity, time/time a rate
  size_t slash = u.find('/');
  if (slash == std::string::npos || slash == 0) return false;
  std::string da, db;
  double sa, sb;
  if (!unit_info(u.substr(0, slash), da, sa) || !unit_info(u.substr(slash + 1), db, sb)) return false;
  if (db != "time" || (da != "length" && da != "time")) return false;
  dim = da == "length" ? "velocity" : "rate";
  scale = sa / sb;
  return true;
}

// "value unit" in `unit`: the value as written when the units agree, else
// converted within one dimension (to_double_amount, Vexpp_node.cc:297-313)
double amount(const std::string &text, const std::string &unit, bool integer) {
  double v;
  char u[256] = {0};
  int n;
  if (integer) {
    int iv;
    n = std::sscanf(text.c_str(), "%d %255s", &iv, u);
    v = iv;
  } else {
    n = std::sscanf(text.c_str(), "%lf %255s", &v, u);
  }
  if (n != 2) throw std::runtime_error("vex: '" + text + "' is not a value with a unit");
  if (unit == u) return v;
  std::string d1, d2;
  double s1, s2;
  if (!unit_info(unit, d1, s1) || !unit_info(u, d2, s2) || d1 != d2)
    throw std::runtime_error("vex: cannot convert '" + text + "' to " + unit);
  return v * s2 / s1;
}

}  // namespace

int VexNode::to_int_amount(const std::string &unit) const { return (int)amount(str(), unit, true); }
double VexNode::to_double_amount(const std::string &unit) const { return amount(str(), unit, false); }

// ---------------------------------------------------------------- scanner

namespace {

enum Tok { T_EOF = 0, T_IDENT, T_COLON, T_SEMI, T_EQ, T_DOLLAR, T_DEF, T_ENDDEF, T_SCAN, T_ENDSCAN, T_REF };

struct Token {
  Tok t;
  std::string text;
  int line;
};

// Characters of an identifier token: anything but & $ * : ; = and white space.
inline bool ident_char(char c) {
  return !(c == '&' || c == '$' || c == '*' || c == ':' || c == ';' || c == '=' || c == '\t' || c == '\n' ||
           c == '\r' || c == ' ');
}
// The scanner's line-end class is the bracket expression [(\r\n)\n]: it
// holds '(' and ')' as well as CR and LF.
inline bool endl_char(char c) { return c == '(' || c == ')' || c == '\r' || c == '\n'; }

class Scanner {
 public:
  explicit Scanner(const std::string &t) : s_(t) {}

  Token next() {
    for (;;) {
      if (literal_) {
        skip_literal();
        continue;
      }
      if (p_ >= s_.size()) return {T_EOF, "", line_};
      char c = s_[p_];
      size_t lit = match_literal_marker("start_literal");
      if (lit) {
        p_ += lit;
        literal_ = true;
        continue;
      }
      if (c == ':') return single(T_COLON);
      if (c == ';') return single(T_SEMI);
      if (c == '=') return single(T_EQ);
      if (c == '$') return single(T_DOLLAR);
      // longest of: an identifier run, a quoted string, a keyword (ties go
      // to the earlier rule: keywords, line end, identifier, quoted string)
      size_t id = 0;
      while (p_ + id < s_.size() && ident_char(s_[p_ + id])) id++;
      size_t q = quoted_length();
      if (id > 0 || q > 0) {
        if (id == 1 && endl_char(c) && q == 0) {  // a lone '(' or ')': a line end
          p_++;
          line_++;
          continue;
        }
        if (q > id) {
          std::string text = s_.substr(p_ + 1, q - 2);
          p_ += q;
          return {T_IDENT, text, line_};
        }
        std::string text = s_.substr(p_, id);
        p_ += id;
        if (text == "def") return {T_DEF, text, line_};
        if (text == "enddef") return {T_ENDDEF, text, line_};
        if (text == "scan") return {T_SCAN, text, line_};
        if (text == "endscan") return {T_ENDSCAN, text, line_};
        if (text == "ref") return {T_REF, text, line_};
        if (text.size() >= 2 && text[0] == '"') text = text.substr(1, text.size() - 2);  // Vexpp_node(const char*)
        return {T_IDENT, text, line_};
      }
      if (c == '\r' || c == '\n') {
        p_++;
        line_++;
        continue;
      }
      if (c == '*') {  // a comment runs to the line end (inclusive)
        size_t e = p_ + 1;
        while (e < s_.size() && s_[e] != '\r' && s_[e] != '\n') e++;
        if (e < s_.size()) {
          p_ = e + 1;
          line_++;
        } else {  // no line end follows: the comment ends at its last '(' or ')', if any
          size_t last = std::string::npos;
          for (size_t k = p_ + 1; k < s_.size(); k++)
            if (s_[k] == '(' || s_[k] == ')') last = k;
          p_ = last == std::string::npos ? p_ + 1 : last + 1;
        }
        continue;
      }
      p_++;  // ' ', '\t', '&': white space
    }
  }

 private:
  const std::string &s_;
  size_t p_ = 0;
  int line_ = 1;
  bool literal_ = false;

  Token single(Tok t) {
    p_++;
    return {t, "", line_};
  }

  // "..." with backslash escapes: its length, or 0
  size_t quoted_length() const {
    if (s_[p_] != '"') return 0;
    size_t k = p_ + 1;
    while (k < s_.size()) {
      if (s_[k] == '\\') {
        if (k + 1 >= s_.size()) return 0;
        k += 2;
        continue;
      }
      if (s_[k] == '"') return k + 1 - p_;
      k++;
    }
    return 0;
  }

  // name "(" [ \t]* ")" [ \t]* ";" at the current position: its length, or 0
  size_t match_literal_marker(const char *name) const {
    size_t n = std::strlen(name);
    if (s_.compare(p_, n, name) != 0) return 0;
    size_t k = p_ + n;
    if (k >= s_.size() || s_[k] != '(') return 0;
    k++;
    while (k < s_.size() && (s_[k] == ' ' || s_[k] == '\t')) k++;
    if (k >= s_.size() || s_[k] != ')') return 0;
    k++;
    while (k < s_.size() && (s_[k] == ' ' || s_[k] == '\t')) k++;
    if (k >= s_.size() || s_[k] != ';') return 0;
    return k + 1 - p_;
  }

  // Inside start_literal() ... end_literal(): the body is skipped a line at a
  // time; the literal ends only where the rest of a line is exactly the end
  // marker (anything longer is taken as body by the longest-match rule).
  void skip_literal() {
    if (p_ >= s_.size()) {
      literal_ = false;
      return;
    }
    size_t e = p_;
    while (e < s_.size() && s_[e] != '\r' && s_[e] != '\n') e++;
    size_t m = match_literal_marker("end_literal");
    if (m && p_ + m == e) {
      p_ = e;
      literal_ = false;
      return;
    }
    p_ = e;
    if (p_ < s_.size()) {
      p_++;
      line_++;
    }
  }
};

// ---------------------------------------------------------------- grammar

class Parser {
 public:
  explicit Parser(const std::string &text) : sc_(text) { adv(); }

  VexNode vex() {
    VexNode root;
    root.kind = VexNode::DICT;
    // header: IDENT = IDENT ;
    std::string key = expect_ident("VEX_rev");
    expect(T_EQ, "=");
    VexNode rev;
    rev.s = expect_ident("revision");
    expect(T_SEMI, ";");
    bool any = false;
    while (tok_.t == T_DOLLAR) {
      adv();
      std::string name = expect_ident("block name");
      expect(T_SEMI, ";");
      root.dict.emplace(name, block_content());
      any = true;
    }
    if (!any || tok_.t != T_EOF) fail("a $BLOCK");
    root.dict.emplace(key, rev);
    return root;
  }

 private:
  Scanner sc_;
  Token tok_;

  void adv() { tok_ = sc_.next(); }
  [[noreturn]] void fail(const char *what) {
    throw std::runtime_error(std::string("vex: syntax error, expected ") + what + " in line " +
                             std::to_string(tok_.line));
  }
  void expect(Tok t, const char *what) {
    if (tok_.t != t) fail(what);
    adv();
  }
  std::string expect_ident(const char *what) {
    if (tok_.t != T_IDENT) fail(what);
    std::string s = tok_.text;
    adv();
    return s;
  }
  // word: IDENT+, joined by single spaces
  std::string word(const char *what) {
    std::string w = expect_ident(what);
    while (tok_.t == T_IDENT) {
      w += " ";
      w += tok_.text;
      adv();
    }
    return w;
  }

  VexNode block_content() {
    VexNode d = lines();
    while (tok_.t == T_DEF || tok_.t == T_SCAN) {
      bool is_def = tok_.t == T_DEF;
      adv();
      std::string name = word("a name");
      expect(T_SEMI, ";");
      VexNode body = lines();
      expect(is_def ? T_ENDDEF : T_ENDSCAN, is_def ? "enddef" : "endscan");
      expect(T_SEMI, ";");
      d.dict.emplace(name, std::move(body));
    }
    return d;
  }

  VexNode lines() {
    VexNode d;
    d.kind = VexNode::DICT;
    while (tok_.t == T_REF || tok_.t == T_IDENT) {
      std::string key;
      if (tok_.t == T_REF) {
        adv();
        expect(T_DOLLAR, "$");
        key = word("a block name");
      } else {
        key = word("a keyword");
      }
      expect(T_EQ, "=");
      d.dict.emplace(key, value());
      expect(T_SEMI, ";");
    }
    return d;
  }

  // value: [word] (':' [word])*  -- a string, or a list once a ':' is seen
  VexNode value() {
    VexNode v;
    if (tok_.t == T_IDENT) v.s = word("a value");
    while (tok_.t == T_COLON) {
      adv();
      if (v.kind == VexNode::STR) {
        VexNode first = v;
        v = VexNode();
        v.kind = VexNode::LIST;
        v.list.push_back(first);
      }
      VexNode item;
      if (tok_.t == T_IDENT) item.s = word("a value");
      v.list.push_back(item);
    }
    return v;
  }
};

}  // namespace

VexNode parse_vex(const std::string &text) { return Parser(text).vex(); }

// ---------------------------------------------------------------- dates

VexDate::VexDate(const std::string &text) {
  std::sscanf(text.c_str(), "%dy%dd%dh%dm%ds", &year, &day, &hour, &minute, &second);
}

void VexDate::normalize() {
  minute += second / 60;
  second %= 60;
  hour += minute / 60;
  minute %= 60;
  day += hour / 24;
  hour %= 24;
  // Date::normalize's leap-year test (year % 100 != 0 && year % 400 == 0)
  // never holds, so its years have 365 days
  year += day / 365;
  day %= 365;
}

VexDate VexDate::plus_seconds(int sec) const {
  VexDate r = *this;
  r.second += sec;
  r.normalize();
  return r;
}

bool VexDate::operator<(const VexDate &o) const {
  VexDate a = *this, b = o;
  a.normalize();
  b.normalize();
  if (a.year != b.year) return a.year < b.year;
  if (a.day != b.day) return a.day < b.day;
  if (a.hour != b.hour) return a.hour < b.hour;
  if (a.minute != b.minute) return a.minute < b.minute;
  return a.second < b.second;
}

bool VexDate::operator==(const VexDate &o) const { return !(*this < o) && !(o < *this); }

std::string VexDate::to_string() const {
  char b[64];
  std::snprintf(b, sizeof b, "%04dy%03dd%02dh%02dm%02ds", year, day, hour, minute, second);
  return b;
}

// ---------------------------------------------------------------- queries

const VexNode &Vex::block(const std::string &name) const {
  const VexNode *b = root_.get(name);
  if (!b) throw std::runtime_error("vex: no $" + name + " block");
  return *b;
}

const VexNode *Vex::def(const std::string &blk, const std::string &name) const {
  const VexNode *b = root_.get(blk);
  return b ? b->get(name) : nullptr;
}

std::vector<std::string> Vex::scans() const {
  std::vector<std::string> out;
  for (const auto &kv : block("SCHED").dict) out.push_back(kv.first);
  return out;
}

std::string Vex::mode(const std::string &scan) const {
  const VexNode *s = def("SCHED", scan);
  if (!s || !s->get("mode")) throw std::runtime_error("vex: scan " + scan + " has no mode");
  return s->get("mode")->str();
}

std::string Vex::start_time_of_scan(const std::string &scan) const {
  const VexNode *s = def("SCHED", scan);
  if (!s || !s->get("start")) throw std::runtime_error("vex: scan " + scan + " has no start");
  return s->get("start")->str();
}

// start + the longest station duration ("%d sec" of field 2)
std::string Vex::stop_time_of_scan(const std::string &scan) const {
  const VexNode *s = def("SCHED", scan);
  std::string start = start_time_of_scan(scan);
  int dur = 0;
  for (const VexNode *st : s->all("station")) {
    int d = 0;
    if (std::sscanf(st->at(2).str().c_str(), "%d sec", &d) == 1 && d > dur) dur = d;
  }
  return VexDate(start).plus_seconds(dur).to_string();
}

std::string Vex::start_time_of_experiment() const {
  std::string r;
  for (const auto &kv : block("SCHED").dict) {
    const VexNode *st = kv.second.get("start");
    if (!st) continue;
    if (r.empty() || r > st->str()) r = st->str();
  }
  return r;
}

std::string Vex::stop_time_of_experiment() const {
  std::string r;
  for (const auto &kv : block("SCHED").dict) {
    std::string cur = stop_time_of_scan(kv.first);
    if (r.empty() || r < cur) r = cur;
  }
  return r;
}

std::string Vex::scan_name(const VexDate &t) const {
  for (const auto &kv : block("SCHED").dict)
    if (t >= start_of_scan(kv.first) && t < stop_of_scan(kv.first)) return kv.first;
  return std::string();
}

int Vex::n_sources(const std::string &scan) const {
  const VexNode *s = def("SCHED", scan);
  return s ? (int)s->all("source").size() : 0;
}

std::string Vex::section(const std::string &sec, const std::string &mode, const std::string &station) const {
  const VexNode *m = def("MODE", mode);
  if (!m) return std::string();
  for (const VexNode *ref : m->all(sec)) {
    if (ref->kind != VexNode::LIST) continue;
    for (size_t i = 1; i < ref->list.size(); i++)
      if (ref->list[i].kind == VexNode::STR && ref->list[i].s == station) return ref->list[0].s;
  }
  return std::string();
}

char Vex::polarisation(const std::string &if_node, const std::string &if_ref) const {
  const VexNode *d = def("IF", if_node);
  if (!d) return ' ';
  for (const auto &kv : d->dict) {
    const VexNode &v = kv.second;
    if (v.kind == VexNode::LIST && v.list.size() > 2 && v.list[0].s == if_ref) return v.list[2].to_char();
  }
  return ' ';
}

}  // namespace sfxc

// VEX files (the observation schedule: stations, modes, frequencies, scans)
// parsed into the tree the reference's parser builds
// (sfxc/lib/vex_parser/vex_parser/src/vex_parser.yy, vex_scanner.ll) and the
// queries its Vex class answers over that tree (src/Vex++.cc).
//
// Tree shape: the file, each $BLOCK, each `def` and each `scan` is a
// dictionary whose keys are kept sorted; a key given more than once keeps
// all its values in file order.  `key = a : b : c;` is a list of strings,
// `key = a;` a string, `ref $X = a : b;` the key X.  Words of several tokens
// are joined by one space ("4974.49 MHz"), '&' counts as white space, '*'
// starts a comment, quoted strings lose their quotes.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace sfxc {

struct VexNode {
  enum Kind { STR = 0, LIST, DICT };
  Kind kind = STR;
  std::string s;
  std::vector<VexNode> list;
  std::multimap<std::string, VexNode> dict;

  // the first value of key in a dictionary, or nullptr
  const VexNode *get(const std::string &key) const;
  // every value of key, in file order
  std::vector<const VexNode *> all(const std::string &key) const;
  // item i of a list (an error for a string or out of range)
  const VexNode &at(size_t i) const;
  size_t size() const { return kind == LIST ? list.size() : kind == DICT ? dict.size() : 0; }
  const std::string &str() const;  // a string's text (an error for a list or dictionary)
  // Vexpp_node::to_int / to_double (leading number), to_*_amount (a number and
  // a unit, converted to `unit` by the scale table of Vexpp_node.cc:174-260)
  int to_int() const;
  double to_double() const;
  int to_int_amount(const std::string &unit) const;
  double to_double_amount(const std::string &unit) const;
  char to_char() const { return str().empty() ? '\0' : str()[0]; }
};

// Parses VEX text; throws std::runtime_error("vex: ... line N") on a syntax error.
VexNode parse_vex(const std::string &text);

// Vexpp_node::Date: "2024y123d12h34m56s" fields (sscanf semantics: a
// missing field stays 0), compared after normalisation.
struct VexDate {
  int year = 0, day = 0, hour = 0, minute = 0, second = 0;
  VexDate() {}
  explicit VexDate(const std::string &text);
  VexDate plus_seconds(int sec) const;
  void normalize();
  bool operator<(const VexDate &o) const;
  bool operator==(const VexDate &o) const;
  bool operator>=(const VexDate &o) const { return !(*this < o); }
  std::string to_string() const;
  // milliseconds since midnight of its own day (Date::to_miliseconds())
  int64_t ms_of_day() const { return 1000LL * (second + 60LL * (minute + 60LL * hour)); }
};

// The Vex class's queries (sfxc/lib/vex_parser/vex_parser/src/Vex++.cc).
class Vex {
 public:
  Vex() {}
  explicit Vex(VexNode root) : root_(std::move(root)) {}
  const VexNode &root() const { return root_; }
  // a block ($FREQ, $SCHED, ...) or one def of it; throws when missing
  const VexNode &block(const std::string &name) const;
  const VexNode *def(const std::string &block, const std::string &name) const;

  std::vector<std::string> scans() const;  // keys of $SCHED, sorted
  std::string mode(const std::string &scan) const;
  std::string start_time_of_experiment() const;
  std::string stop_time_of_experiment() const;
  std::string start_time_of_scan(const std::string &scan) const;
  std::string stop_time_of_scan(const std::string &scan) const;
  VexDate start_of_scan(const std::string &scan) const { return VexDate(start_time_of_scan(scan)); }
  VexDate stop_of_scan(const std::string &scan) const { return VexDate(stop_time_of_scan(scan)); }
  std::string scan_name(const VexDate &t) const;  // the scan holding t, or ""
  int n_sources(const std::string &scan) const;
  // the def of a $MODE section (FREQ, IF, BBC, TRACKS, BITSTREAMS, THREADS)
  // that names `station`, or ""
  std::string section(const std::string &section, const std::string &mode, const std::string &station) const;
  // polarisation of if_ref in $IF def if_node, or ' '
  char polarisation(const std::string &if_node, const std::string &if_ref) const;

 private:
  VexNode root_;
};

}  // namespace sfxc

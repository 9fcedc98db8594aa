// JSON values for the correlator control file, read with the rules of the
// JSON reader the reference links (sfxc/lib/jsoncpp: objects with sorted
// keys, '//' and C comments allowed, numbers without '.', 'e', 'E', '+' or an
// inner '-' are integers) and the conversions of its Value class
// (json_value.cpp:662-802: asInt truncates reals, asBool is true for a
// non-empty string or container; a conversion it refuses throws).
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace sfxc {

class Json {
 public:
  enum Type { NUL = 0, INT, REAL, STRING, BOOL, ARRAY, OBJECT };

  Json() {}
  static Json parse(const std::string &text);  // throws std::runtime_error

  Type type() const { return t_; }
  bool is_null() const { return t_ == NUL; }
  // member lookup; a missing member (or a lookup in a non-object) reads as null
  const Json &operator[](const std::string &key) const;
  const Json &operator[](size_t i) const;
  size_t size() const { return t_ == ARRAY ? arr_.size() : t_ == OBJECT ? obj_.size() : 0; }
  const std::map<std::string, Json> &members() const { return obj_; }
  const std::vector<Json> &items() const { return arr_; }

  std::string as_string() const;
  int as_int() const;
  int64_t as_int64() const { return t_ == INT ? i_ : (int64_t)as_double(); }
  double as_double() const;
  bool as_bool() const;

  // building (for defaults filled in after reading)
  void set(const std::string &key, Json v);
  void append(Json v);
  static Json of_string(const std::string &s);
  static Json of_int(int64_t v);
  static Json of_double(double v);
  static Json of_bool(bool v);

  std::string dump() const;  // compact JSON text

 private:
  Type t_ = NUL;
  int64_t i_ = 0;
  double d_ = 0;
  bool b_ = false;
  std::string s_;
  std::vector<Json> arr_;
  std::map<std::string, Json> obj_;
  friend class JsonReader;
};

}  // namespace sfxc

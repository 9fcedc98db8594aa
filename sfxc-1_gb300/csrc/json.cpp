// JSON reader and values; see json.hpp.
#include "json.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>

namespace sfxc {

namespace {
const Json &null_json() {
  static const Json n;
  return n;
}
}  // namespace

class JsonReader {
 public:
  explicit JsonReader(const std::string &t) : s_(t) {}

  Json document() {
    Json v = value();
    skip();
    if (p_ != s_.size()) fail("extra text after the document");
    return v;
  }

 private:
  const std::string &s_;
  size_t p_ = 0;

  [[noreturn]] void fail(const std::string &what) const {
    int line = 1;
    for (size_t k = 0; k < p_ && k < s_.size(); k++) line += s_[k] == '\n';
    throw std::runtime_error("ctrl file: " + what + " in line " + std::to_string(line));
  }

  void skip() {
    for (;;) {
      while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\r' || s_[p_] == '\n')) p_++;
      if (p_ + 1 < s_.size() && s_[p_] == '/' && s_[p_ + 1] == '/') {
        while (p_ < s_.size() && s_[p_] != '\n' && s_[p_] != '\r') p_++;
      } else if (p_ + 1 < s_.size() && s_[p_] == '/' && s_[p_ + 1] == '*') {
        size_t e = s_.find("*/", p_ + 2);
        if (e == std::string::npos) fail("unterminated comment");
        p_ = e + 2;
      } else {
        return;
      }
    }
  }

  Json value() {
    skip();
    if (p_ >= s_.size()) fail("a value");
    char c = s_[p_];
    Json v;
    if (c == '{') {
      p_++;
      v.t_ = Json::OBJECT;
      skip();
      if (p_ < s_.size() && s_[p_] == '}') {
        p_++;
        return v;
      }
      for (;;) {
        skip();
        if (p_ >= s_.size() || s_[p_] != '"') fail("a member name");
        std::string key = string_body();
        skip();
        if (p_ >= s_.size() || s_[p_] != ':') fail("':'");
        p_++;
        v.obj_[key] = value();
        skip();
        if (p_ < s_.size() && s_[p_] == ',') {
          p_++;
          continue;
        }
        if (p_ < s_.size() && s_[p_] == '}') {
          p_++;
          return v;
        }
        fail("',' or '}'");
      }
    }
    if (c == '[') {
      p_++;
      v.t_ = Json::ARRAY;
      skip();
      if (p_ < s_.size() && s_[p_] == ']') {
        p_++;
        return v;
      }
      for (;;) {
        v.arr_.push_back(value());
        skip();
        if (p_ < s_.size() && s_[p_] == ',') {
          p_++;
          continue;
        }
        if (p_ < s_.size() && s_[p_] == ']') {
          p_++;
          return v;
        }
        fail("',' or ']'");
      }
    }
    if (c == '"') {
      v.t_ = Json::STRING;
      v.s_ = string_body();
      return v;
    }
    if (s_.compare(p_, 4, "true") == 0) {
      p_ += 4;
      v.t_ = Json::BOOL;
      v.b_ = true;
      return v;
    }
    if (s_.compare(p_, 5, "false") == 0) {
      p_ += 5;
      v.t_ = Json::BOOL;
      return v;
    }
    if (s_.compare(p_, 4, "null") == 0) {
      p_ += 4;
      return v;
    }
    if (c == '-' || (c >= '0' && c <= '9')) return number();
    fail("a value");
  }

  // A number token runs over digits and . e E + -; it is an integer when it
  // holds none of '.', 'e', 'E', '+' and no '-' but a leading one, and fits.
  Json number() {
    size_t b = p_;
    while (p_ < s_.size()) {
      char c = s_[p_];
      if ((c >= '0' && c <= '9') || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-')
        p_++;
      else
        break;
    }
    std::string tok = s_.substr(b, p_ - b);
    bool real = false;
    for (size_t k = 0; k < tok.size(); k++)
      if (tok[k] == '.' || tok[k] == 'e' || tok[k] == 'E' || tok[k] == '+' || (tok[k] == '-' && k > 0)) real = true;
    Json v;
    if (!real) {
      bool neg = tok[0] == '-';
      size_t k = neg ? 1 : 0;
      if (k == tok.size()) fail("'" + tok + "' is not a number");
      uint64_t val = 0;
      bool fits = true;
      for (; k < tok.size(); k++) {
        if (tok[k] < '0' || tok[k] > '9') fail("'" + tok + "' is not a number");
        if (val >= (neg ? 2147483648ULL : 4294967295ULL) / 10) fits = false;
        if (!fits) break;
        val = val * 10 + (uint64_t)(tok[k] - '0');
      }
      if (fits) {
        v.t_ = Json::INT;
        v.i_ = neg ? -(int64_t)val : (int64_t)val;
        return v;
      }
    }
    char *end = nullptr;
    double d = std::strtod(tok.c_str(), &end);
    if (!end || *end) fail("'" + tok + "' is not a number");
    v.t_ = Json::REAL;
    v.d_ = d;
    return v;
  }

  std::string string_body() {
    std::string out;
    p_++;  // opening quote
    while (p_ < s_.size()) {
      char c = s_[p_++];
      if (c == '"') return out;
      if (c != '\\') {
        out += c;
        continue;
      }
      if (p_ >= s_.size()) break;
      char e = s_[p_++];
      switch (e) {
        case '"': out += '"'; break;
        case '/': out += '/'; break;
        case '\\': out += '\\'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          if (p_ + 4 > s_.size()) fail("a \\u escape");
          unsigned cp = (unsigned)std::strtoul(s_.substr(p_, 4).c_str(), nullptr, 16);
          p_ += 4;
          if (cp < 0x80) {
            out += (char)cp;
          } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
          } else {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
          }
          break;
        }
        default: fail("a string escape");
      }
    }
    fail("an unterminated string");
  }
};

Json Json::parse(const std::string &text) { return JsonReader(text).document(); }

const Json &Json::operator[](const std::string &key) const {
  if (t_ != OBJECT) return null_json();
  auto it = obj_.find(key);
  return it == obj_.end() ? null_json() : it->second;
}

const Json &Json::operator[](size_t i) const {
  if (t_ != ARRAY || i >= arr_.size()) return null_json();
  return arr_[i];
}

std::string Json::as_string() const {
  switch (t_) {
    case NUL: return "";
    case STRING: return s_;
    case BOOL: return b_ ? "true" : "false";
    default: throw std::runtime_error("ctrl file: a value is not convertible to a string");
  }
}

int Json::as_int() const {
  switch (t_) {
    case NUL: return 0;
    case INT: return (int)i_;
    case REAL:
      if (!(d_ >= -2147483648.0 && d_ <= 2147483647.0)) throw std::runtime_error("ctrl file: a number out of range");
      return (int)d_;
    case BOOL: return b_ ? 1 : 0;
    default: throw std::runtime_error("ctrl file: a value is not convertible to an integer");
  }
}

double Json::as_double() const {
  switch (t_) {
    case NUL: return 0;
    case INT: return (double)i_;
    case REAL: return d_;
    case BOOL: return b_ ? 1 : 0;
    default: throw std::runtime_error("ctrl file: a value is not convertible to a number");
  }
}

bool Json::as_bool() const {
  switch (t_) {
    case NUL: return false;
    case INT: return i_ != 0;
    case REAL: return d_ != 0;
    case BOOL: return b_;
    case STRING: return !s_.empty();
    case ARRAY: return !arr_.empty();
    case OBJECT: return !obj_.empty();
  }
  return false;
}

void Json::set(const std::string &key, Json v) {
  if (t_ == NUL) t_ = OBJECT;
  if (t_ != OBJECT) throw std::runtime_error("ctrl file: member set on a value that is not an object");
  obj_[key] = std::move(v);
}

void Json::append(Json v) {
  if (t_ == NUL) t_ = ARRAY;
  if (t_ != ARRAY) throw std::runtime_error("ctrl file: item appended to a value that is not an array");
  arr_.push_back(std::move(v));
}

Json Json::of_string(const std::string &s) {
  Json v;
  v.t_ = STRING;
  v.s_ = s;
  return v;
}
Json Json::of_int(int64_t x) {
  Json v;
  v.t_ = INT;
  v.i_ = x;
  return v;
}
Json Json::of_double(double x) {
  Json v;
  v.t_ = REAL;
  v.d_ = x;
  return v;
}
Json Json::of_bool(bool x) {
  Json v;
  v.t_ = BOOL;
  v.b_ = x;
  return v;
}

namespace {
void quote(const std::string &s, std::string &out) {
  out += '"';
  for (unsigned char c : s) {
    if (c == '"' || c == '\\') {
      out += '\\';
      out += (char)c;
    } else if (c < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", c);
      out += b;
    } else {
      out += (char)c;
    }
  }
  out += '"';
}

void dump_to(const Json &v, std::string &out) {
  switch (v.type()) {
    case Json::NUL: out += "null"; break;
    case Json::INT: out += std::to_string((long long)v.as_int64()); break;
    case Json::REAL: {
      char b[40];
      std::snprintf(b, sizeof b, "%.17g", v.as_double());
      out += b;
      break;
    }
    case Json::STRING: quote(v.as_string(), out); break;
    case Json::BOOL: out += v.as_bool() ? "true" : "false"; break;
    case Json::ARRAY: {
      out += '[';
      bool first = true;
      for (const Json &x : v.items()) {
        if (!first) out += ',';
        first = false;
        dump_to(x, out);
      }
      out += ']';
      break;
    }
    case Json::OBJECT: {
      out += '{';
      bool first = true;
      for (const auto &kv : v.members()) {
        if (!first) out += ',';
        first = false;
        quote(kv.first, out);
        out += ':';
        dump_to(kv.second, out);
      }
      out += '}';
      break;
    }
  }
}
}  // namespace

std::string Json::dump() const {
  std::string out;
  dump_to(*this, out);
  return out;
}

}  // namespace sfxc

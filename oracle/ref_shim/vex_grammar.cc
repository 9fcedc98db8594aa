// The reference's VEX scanner and grammar (flex rules of
// sfxc/lib/vex_parser/vex_parser/src/vex_scanner.ll:1-55, bison rules and
// their actions of vex_parser.yy:20-160) restated by hand, because neither
// flex nor bison is available to generate them: yyparse() reads yyin and
// leaves the tree in parse_result, built with the reference's own
// Vexpp_node operations (set_key, join, append) exactly as the grammar's
// actions do.  Linked only into the checker with the reference's Vex++.cc,
// Vexpp_node.cc and Control_parameters.  Test infrastructure only.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "generic.h"

FILE *yyin = NULL, *yyout = NULL;
YYSTYPE parse_result;
int linenr = 0;

void yyerror(char const *s) { std::fprintf(stderr, " == Error: %s\n == In line: %d\n\n", s, linenr); }
void yyrestart(FILE *f) { yyin = f; }
int yylex() { return 0; }

namespace {

enum { IDENT = 1, COLON, SEMICOLON, EQ, DOLLAR, DEF, ENDDEF, SCAN, ENDSCAN, REF, END };

struct Lexeme {
  int kind;
  std::string text;  // IDENT: the matched text, quotes included (Vexpp_node strips them)
  int line;
};

bool is_token_char(char c) { return std::strchr("&$*:;=\t\n\r ", c) == NULL || c == 0; }
bool is_endl_char(char c) { return c == '(' || c == ')' || c == '\r' || c == '\n'; }

// "name(" [ \t]* ")" [ \t]* ";" at s[i]: length or 0
size_t literal_marker(const std::string &s, size_t i, const char *name) {
  size_t n = std::strlen(name);
  if (s.compare(i, n, name) != 0) return 0;
  size_t k = i + n;
  if (k >= s.size() || s[k] != '(') return 0;
  for (k++; k < s.size() && (s[k] == ' ' || s[k] == '\t'); k++) {
  }
  if (k >= s.size() || s[k] != ')') return 0;
  for (k++; k < s.size() && (s[k] == ' ' || s[k] == '\t'); k++) {
  }
  if (k >= s.size() || s[k] != ';') return 0;
  return k + 1 - i;
}

// The flex scanner: at each position the longest match of the rules, ties to
// the earlier rule; the literal start condition eats whole lines.
std::vector<Lexeme> scan_all(const std::string &s) {
  std::vector<Lexeme> out;
  size_t i = 0;
  int line = 1;
  bool literal = false;
  while (i < s.size()) {
    if (literal) {
      size_t e = i;
      while (e < s.size() && s[e] != '\r' && s[e] != '\n') e++;
      size_t m = literal_marker(s, i, "end_literal");
      if (e == i) {  // a line end ({ENDL} in the literal condition)
        i++;
        line++;
        continue;
      }
      if (m && i + m == e) literal = false;  // the end marker ties with the body rule and wins
      i = e;
      continue;
    }
    size_t lit = literal_marker(s, i, "start_literal");
    if (lit) {
      i += lit;
      literal = true;
      continue;
    }
    char c = s[i];
    int single = c == ':' ? COLON : c == ';' ? SEMICOLON : c == '=' ? EQ : c == '$' ? DOLLAR : 0;
    if (single) {
      Lexeme l = {single, std::string(), line};
      out.push_back(l);
      i++;
      continue;
    }
    size_t tok = 0;
    while (i + tok < s.size() && is_token_char(s[i + tok])) tok++;
    size_t quoted = 0;
    if (c == '"') {
      size_t k = i + 1;
      while (k < s.size() && s[k] != '"') {
        if (s[k] == '\\') {
          if (k + 1 >= s.size()) break;
          k++;
        }
        k++;
      }
      if (k < s.size() && s[k] == '"') quoted = k + 1 - i;
    }
    if (tok == 1 && is_endl_char(c) && quoted == 0) {  // {ENDL} is listed before {TOKEN}+
      i++;
      line++;
      continue;
    }
    if (tok > 0 || quoted > 0) {
      size_t n = quoted > tok ? quoted : tok;
      std::string text = s.substr(i, n);
      int kind = IDENT;
      if (quoted <= tok) {  // keywords only when the identifier rule is the match
        if (text == "def") kind = DEF;
        else if (text == "enddef") kind = ENDDEF;
        else if (text == "scan") kind = SCAN;
        else if (text == "endscan") kind = ENDSCAN;
        else if (text == "ref") kind = REF;
      }
      Lexeme l = {kind, text, line};
      out.push_back(l);
      i += n;
      continue;
    }
    if (c == '\r' || c == '\n') {
      i++;
      line++;
      continue;
    }
    if (c == '*') {
      size_t e = i + 1;
      while (e < s.size() && s[e] != '\r' && s[e] != '\n') e++;
      if (e < s.size()) {
        i = e + 1;
        line++;
      } else {
        size_t last = std::string::npos;
        for (size_t k = i + 1; k < s.size(); k++)
          if (s[k] == '(' || s[k] == ')') last = k;
        i = last == std::string::npos ? i + 1 : last + 1;
      }
      continue;
    }
    i++;  // [ \t&]+, or a character no rule matches (flex echoes it)
  }
  Lexeme end = {END, std::string(), line};
  out.push_back(end);
  return out;
}

struct Grammar {
  std::vector<Lexeme> lx;
  size_t p;
  bool ok;

  int kind() const { return lx[p].kind; }
  void error() {
    if (ok) {
      linenr = lx[p].line;
      yyerror("syntax error");
    }
    ok = false;
  }
  bool take(int k) {
    if (kind() != k) {
      error();
      return false;
    }
    p++;
    return true;
  }

  // word: IDENT | word IDENT  { key = $1 + " " + $2; $$ = YYSTYPE(key) }
  YYSTYPE word() {
    if (kind() != IDENT) {
      error();
      return YYSTYPE("");
    }
    YYSTYPE w(lx[p++].text.c_str());
    while (kind() == IDENT) {
      YYSTYPE next(lx[p++].text.c_str());
      std::string key = w.to_string() + " " + next.to_string();
      w = YYSTYPE(key.c_str());
    }
    return w;
  }

  // value: word | (empty) | value COLON word | value COLON
  YYSTYPE value() {
    YYSTYPE v = kind() == IDENT ? word() : YYSTYPE("");
    while (ok && kind() == COLON) {
      p++;
      if (v.get_type() == YYSTYPE::STRING) {
        YYSTYPE first = v;
        v = YYSTYPE(YYSTYPE::ARRAY);
        v.append(first);
      }
      if (kind() == IDENT)
        v.append(word());
      else
        v.append(YYSTYPE(""));
    }
    return v;
  }

  // block_lines: (empty) | block_lines block_line
  YYSTYPE block_lines() {
    YYSTYPE lines(YYSTYPE::DICT);
    while (ok && (kind() == REF || kind() == IDENT)) {
      YYSTYPE line(YYSTYPE::DICT);
      YYSTYPE key;
      if (kind() == REF) {
        p++;
        if (!take(DOLLAR)) break;
        key = word();
      } else {
        key = word();
      }
      if (!take(EQ)) break;
      YYSTYPE v = value();
      if (!take(SEMICOLON)) break;
      line.set_key(key.to_string(), v);
      lines.join(line);
    }
    return lines;
  }

  // block_content: block_lines | block_content def_block | block_content scan_block
  YYSTYPE block_content() {
    YYSTYPE content = block_lines();
    while (ok && (kind() == DEF || kind() == SCAN)) {
      bool def = kind() == DEF;
      p++;
      YYSTYPE name = word();
      if (!take(SEMICOLON)) break;
      YYSTYPE body = block_lines();
      if (!take(def ? ENDDEF : ENDSCAN) || !take(SEMICOLON)) break;
      YYSTYPE one(YYSTYPE::DICT);
      one.set_key(name.to_string(), body);
      content.join(one);
    }
    return content;
  }

  // vex: vex_header blocks   { $$ = $3; $$.join($2); }
  bool vex() {
    if (kind() != IDENT) {
      error();
      return false;
    }
    YYSTYPE key(lx[p++].text.c_str());
    if (!take(EQ) || kind() != IDENT) {
      error();
      return false;
    }
    YYSTYPE rev(lx[p++].text.c_str());
    if (!take(SEMICOLON)) return false;
    YYSTYPE header(YYSTYPE::DICT);
    header.set_key(key.to_string(), rev);
    YYSTYPE blocks(YYSTYPE::DICT);
    int n = 0;
    while (ok && kind() == DOLLAR) {
      p++;
      if (kind() != IDENT) {
        error();
        return false;
      }
      YYSTYPE name(lx[p++].text.c_str());
      if (!take(SEMICOLON)) return false;
      YYSTYPE content = block_content();
      YYSTYPE block(YYSTYPE::DICT);
      block.set_key(name.to_string(), content);
      blocks.join(block);
      n++;
    }
    if (!ok || n == 0 || kind() != END) {
      error();
      return false;
    }
    blocks.join(header);
    parse_result = blocks;
    return true;
  }
};

}  // namespace

int yyparse() {
  std::string text;
  if (yyin) {
    char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, yyin)) > 0) text.append(buf, n);
  }
  Grammar g;
  g.lx = scan_all(text);
  g.p = 0;
  g.ok = true;
  linenr = 1;
  return g.vex() ? 0 : 1;
}

// sdl.hpp -- the POV-Ray scene-description subset CueMol writes, as the two
// readers (pov_scene_reader.cpp: the .pov viewing setup; mesh2_reader.cpp:
// the .inc geometry) need it: a tokenizer, numeric / vector values with
// scalar broadcast, and the expression grammar of #declare values, vectors
// and block arguments.  Not a POV-Ray interpreter: macros are not expanded
// and unknown names evaluate to nothing (a zero of no components).
//
// Behaviour follows the reference readers (src/bench/pov/pov_lexer.cpp,
// pov_scene_reader.cpp:148-244, src/bench/geom/mesh2_reader.cpp:85-148):
// `//` and `/* */` comments, numbers by strtod over [digits][.digits]
// [e[+-]digits], identifiers [A-Za-z_][A-Za-z0-9_]*, "strings", every other
// character one punctuation token; sums of products of unary terms, vectors
// of at most four components, component-wise arithmetic with scalar
// broadcast and division by zero giving zero.
#pragma once

#include <cstddef>
#include <map>
#include <string>
#include <vector>

namespace umbreon {
namespace sdl {

enum class Kind : unsigned char { Number, Name, Text, Symbol, Eof };

struct Tok {
  Kind kind = Kind::Eof;
  double number = 0.0;
  std::string text;  // name, string body, or the punctuation character
  int line = 1;
};

std::vector<Tok> lex(const std::string& src);

// A scalar (n = 1) or a 2..4 component vector; n = 0 is "no value".
struct Val {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  int n = 0;
  // component i, a scalar standing for all four
  double at(int i) const { return n == 0 ? 0.0 : n == 1 ? v[0] : (i < n ? v[i] : 0.0); }
  static Val scalar(double x) {
    Val r;
    r.v[0] = x;
    r.n = 1;
    return r;
  }
};

// a op b component-wise ('+', '-', '*', '/'); two scalars give a scalar
Val combine(const Val& a, const Val& b, char op);

using Vars = std::map<std::string, Val>;

// A token stream with a read position, the grammar's evaluator and the block
// helpers both readers use.
class Stream {
 public:
  explicit Stream(std::vector<Tok> toks) : t_(std::move(toks)) {
    if (t_.empty() || t_.back().kind != Kind::Eof) t_.push_back(Tok{});
  }

  std::size_t pos = 0;

  const Tok& at(std::size_t k) const { return t_[k < t_.size() ? k : t_.size() - 1]; }
  const Tok& cur() const { return at(pos); }
  bool done() const { return cur().kind == Kind::Eof; }
  void next() {
    if (!done()) ++pos;
  }
  bool isSym(std::size_t k, char c) const { return at(k).kind == Kind::Symbol && at(k).text[0] == c; }
  bool sym(char c) const { return isSym(pos, c); }
  bool isName(std::size_t k) const { return at(k).kind == Kind::Name; }
  bool name() const { return isName(pos); }
  bool number() const { return cur().kind == Kind::Number; }
  std::size_t size() const { return t_.size(); }

  // index of the '}' closing the '{' at `open`, or npos when unbalanced
  std::size_t closing(std::size_t open) const;

  // Expression at the cursor (advances past it).  With `calls` a name
  // followed by '(' is one of the math functions (degrees, radians, atan2,
  // atan, tan, sin, cos, sqrt, abs, floor, int, min, max, pow, vlength,
  // vnormalize, vdot, vcross; others give nothing); without, the call's
  // parenthesised tokens are skipped and it gives nothing.
  Val expr(const Vars& vars, bool calls);

  // "( a, b, ... )" at the cursor: the evaluated arguments
  std::vector<Val> arguments(const Vars& vars, bool calls);
  // skip a balanced "( ... )" at the cursor
  void skipParens();
  // skip to just past the next ';' at bracket depth 0, or to a '#' there
  void skipStatement();
  // skip "#macro ... #end" with the cursor on `macro` (nested blocks counted)
  void skipMacro();

 private:
  Val term(const Vars& vars, bool calls);
  Val unary(const Vars& vars, bool calls);
  std::vector<Tok> t_;
};

// "color" keywords of POV's colour syntax
bool isColorKeyword(const std::string& s);

}  // namespace sdl
}  // namespace umbreon

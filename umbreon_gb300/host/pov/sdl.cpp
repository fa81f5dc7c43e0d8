// sdl.cpp -- tokenizer, values and expression grammar shared by the POV
// readers (behaviour as stated in sdl.hpp).
#include "sdl.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace umbreon {
namespace sdl {
namespace {

bool asciiDigit(unsigned char c) { return c >= '0' && c <= '9'; }
bool asciiAlpha(unsigned char c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'); }
bool nameStart(unsigned char c) { return asciiAlpha(c) || c == '_'; }
bool nameChar(unsigned char c) { return nameStart(c) || asciiDigit(c); }
bool space(unsigned char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

Val callFunction(const std::string& fn, const std::vector<Val>& a) {
  auto s = [&](std::size_t i) { return i < a.size() ? a[i].at(0) : 0.0; };
  auto vec3 = [](double x, double y, double z) {
    Val r;
    r.v[0] = x;
    r.v[1] = y;
    r.v[2] = z;
    r.n = 3;
    return r;
  };
  constexpr double kPi = 3.14159265358979323846;
  if (fn == "degrees") return Val::scalar(s(0) * (180.0 / kPi));
  if (fn == "radians") return Val::scalar(s(0) * (kPi / 180.0));
  if (fn == "atan2") return Val::scalar(std::atan2(s(0), s(1)));
  if (fn == "atan") return Val::scalar(std::atan(s(0)));
  if (fn == "tan") return Val::scalar(std::tan(s(0)));
  if (fn == "sin") return Val::scalar(std::sin(s(0)));
  if (fn == "cos") return Val::scalar(std::cos(s(0)));
  if (fn == "sqrt") return Val::scalar(std::sqrt(std::max(0.0, s(0))));
  if (fn == "abs") return Val::scalar(std::fabs(s(0)));
  if (fn == "floor") return Val::scalar(std::floor(s(0)));
  if (fn == "int") return Val::scalar(std::trunc(s(0)));
  if (fn == "min") return Val::scalar(std::min(s(0), s(1)));
  if (fn == "max") return Val::scalar(std::max(s(0), s(1)));
  if (fn == "pow") return Val::scalar(std::pow(s(0), s(1)));
  if (a.empty()) return Val{};
  const Val& p = a[0];
  const double len = std::sqrt(p.at(0) * p.at(0) + p.at(1) * p.at(1) + p.at(2) * p.at(2));
  if (fn == "vlength") return Val::scalar(len);
  if (fn == "vnormalize") return len > 0.0 ? vec3(p.at(0) / len, p.at(1) / len, p.at(2) / len) : vec3(0, 0, 0);
  if (a.size() < 2) return Val{};
  const Val& q = a[1];
  if (fn == "vdot") return Val::scalar(p.at(0) * q.at(0) + p.at(1) * q.at(1) + p.at(2) * q.at(2));
  if (fn == "vcross")
    return vec3(p.at(1) * q.at(2) - p.at(2) * q.at(1), p.at(2) * q.at(0) - p.at(0) * q.at(2),
                p.at(0) * q.at(1) - p.at(1) * q.at(0));
  return Val{};
}

}  // namespace

std::vector<Tok> lex(const std::string& src) {
  std::vector<Tok> out;
  const std::size_t n = src.size();
  int line = 1;
  std::size_t i = 0;
  auto uc = [&](std::size_t k) { return static_cast<unsigned char>(src[k]); };
  while (i < n) {
    const unsigned char c = uc(i);
    if (c == '\n') {
      ++line;
      ++i;
    } else if (space(c)) {
      ++i;
    } else if (c == '/' && i + 1 < n && src[i + 1] == '/') {
      while (i < n && src[i] != '\n') ++i;
    } else if (c == '/' && i + 1 < n && src[i + 1] == '*') {
      std::size_t k = i + 2;
      while (k + 1 < n && !(src[k] == '*' && src[k + 1] == '/')) {
        if (src[k] == '\n') ++line;
        ++k;
      }
      i = k + 1 < n ? k + 2 : n;
    } else if (c == '"') {
      Tok t;
      t.kind = Kind::Text;
      t.line = line;
      std::size_t k = i + 1;
      while (k < n && src[k] != '"') {
        if (src[k] == '\n') ++line;
        t.text.push_back(src[k++]);
      }
      out.push_back(std::move(t));
      i = k < n ? k + 1 : n;
    } else if (asciiDigit(c) || (c == '.' && i + 1 < n && asciiDigit(uc(i + 1)))) {
      std::size_t k = i;
      while (k < n && asciiDigit(uc(k))) ++k;
      if (k < n && src[k] == '.') {
        ++k;
        while (k < n && asciiDigit(uc(k))) ++k;
      }
      if (k < n && (src[k] == 'e' || src[k] == 'E')) {
        std::size_t e = k + 1;
        if (e < n && (src[e] == '+' || src[e] == '-')) ++e;
        if (e < n && asciiDigit(uc(e))) {
          k = e;
          while (k < n && asciiDigit(uc(k))) ++k;
        }
      }
      Tok t;
      t.kind = Kind::Number;
      t.number = std::strtod(src.substr(i, k - i).c_str(), nullptr);
      t.line = line;
      out.push_back(std::move(t));
      i = k;
    } else if (nameStart(c)) {
      std::size_t k = i;
      while (k < n && nameChar(uc(k))) ++k;
      Tok t;
      t.kind = Kind::Name;
      t.text = src.substr(i, k - i);
      t.line = line;
      out.push_back(std::move(t));
      i = k;
    } else {
      Tok t;
      t.kind = Kind::Symbol;
      t.text = std::string(1, src[i]);
      t.line = line;
      out.push_back(std::move(t));
      ++i;
    }
  }
  Tok end;
  end.line = line;
  out.push_back(end);
  return out;
}

Val combine(const Val& a, const Val& b, char op) {
  Val r;
  r.n = (a.n <= 1 && b.n <= 1) ? 1 : std::max(a.n, b.n);
  for (int i = 0; i < r.n; ++i) {
    const double x = a.at(i), y = b.at(i);
    r.v[i] = op == '+' ? x + y : op == '-' ? x - y : op == '*' ? x * y : (y != 0.0 ? x / y : 0.0);
  }
  return r;
}

bool isColorKeyword(const std::string& s) {
  static const char* const kw[] = {"rgb", "rgbf", "rgbt", "rgbft", "srgb", "srgbf", "srgbt", "srgbft"};
  for (const char* k : kw)
    if (s == k) return true;
  return false;
}

std::size_t Stream::closing(std::size_t open) const {
  int depth = 0;
  for (std::size_t k = open; k < t_.size() && t_[k].kind != Kind::Eof; ++k) {
    if (isSym(k, '{')) ++depth;
    else if (isSym(k, '}') && --depth == 0) return k;
  }
  return std::string::npos;
}

Val Stream::unary(const Vars& vars, bool calls) {
  if (sym('-')) {
    next();
    Val v = unary(vars, calls);
    for (int i = 0; i < v.n; ++i) v.v[i] = -v.v[i];
    return v;
  }
  if (sym('+')) {
    next();
    return unary(vars, calls);
  }
  if (sym('(')) {
    next();
    Val v = expr(vars, calls);
    if (sym(')')) next();
    return v;
  }
  if (sym('<')) {
    next();
    Val v;
    while (!sym('>') && !done() && v.n < 4) {
      const Val e = expr(vars, calls);
      v.v[v.n++] = e.n > 0 ? e.v[0] : 0.0;
      if (!sym(',')) break;
      next();
    }
    if (sym('>')) next();
    return v;
  }
  if (number()) {
    const Val v = Val::scalar(cur().number);
    next();
    return v;
  }
  if (name()) {
    const std::string id = cur().text;
    next();
    if (sym('(')) {
      if (!calls) {
        skipParens();
        return Val{};
      }
      return callFunction(id, arguments(vars, calls));
    }
    const auto it = vars.find(id);
    return it != vars.end() ? it->second : Val{};
  }
  return Val{};
}

Val Stream::term(const Vars& vars, bool calls) {
  Val a = unary(vars, calls);
  while (sym('*') || sym('/')) {
    const char op = cur().text[0];
    next();
    a = combine(a, unary(vars, calls), op);
  }
  return a;
}

Val Stream::expr(const Vars& vars, bool calls) {
  Val a = term(vars, calls);
  while (sym('+') || sym('-')) {
    const char op = cur().text[0];
    next();
    a = combine(a, term(vars, calls), op);
  }
  return a;
}

std::vector<Val> Stream::arguments(const Vars& vars, bool calls) {
  std::vector<Val> out;
  if (!sym('(')) return out;
  next();
  if (!sym(')')) {
    out.push_back(expr(vars, calls));
    while (sym(',')) {
      next();
      out.push_back(expr(vars, calls));
    }
  }
  if (sym(')')) next();
  return out;
}

void Stream::skipParens() {
  int depth = 0;
  do {
    if (sym('(')) ++depth;
    else if (sym(')')) --depth;
    next();
  } while (depth > 0 && !done());
}

void Stream::skipStatement() {
  int depth = 0;
  for (; !done(); next()) {
    if (cur().kind != Kind::Symbol) continue;
    const char c = cur().text[0];
    if (c == '{' || c == '(' || c == '[') {
      ++depth;
    } else if (c == '}' || c == ')' || c == ']') {
      if (depth > 0) --depth;
    } else if (depth == 0 && c == ';') {
      next();
      return;
    } else if (depth == 0 && c == '#') {
      return;
    }
  }
}

void Stream::skipMacro() {
  next();  // `macro`
  int depth = 1;
  while (!done() && depth > 0) {
    if (!sym('#')) {
      next();
      continue;
    }
    next();
    if (!name()) continue;
    const std::string& d = cur().text;
    if (d == "macro" || d == "if" || d == "ifdef" || d == "ifndef" || d == "while" || d == "for" || d == "switch")
      ++depth;
    else if (d == "end")
      --depth;
    next();
  }
}

}  // namespace sdl
}  // namespace umbreon

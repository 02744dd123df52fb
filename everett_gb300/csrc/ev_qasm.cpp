// ev_qasm.cpp -- OpenQASM 3 ingress and egress for the engine's op records
// (host C++; the reference's reader and writer are src/qasm/parse.rs,
// emit.rs and gates.rs).
//
// The accepted language, the resulting circuit and every error (message,
// line and column) follow the reference's recursive-descent reader: a
// version line and an include line, both optional; `qubit[n] name;` and
// `bit[n] name;` (the last declaration of each kind wins); gate
// definitions skipped by brace counting; the stdgates.inc 1-qubit names
// (h x y z s t id rx ry rz p phase) and 2-qubit names (cx cnot CX cz swap);
// `ctrl @` / `ctrl(k) @` modifiers; both measurement forms; `if (c[i] == 1)`
// around one statement; `reset` and `barrier` skipped; angle expressions
// over literals, pi and tau with unary minus and + - * /.  An error is
// reported at the position of the token after the one that failed, because
// the reference peeks that token to build the error.
//
// Parsed circuits are returned as op records ready for the run loop
// (`IfClassic` in prefix form), with gate matrices built by the reference's
// constructors (src/gate.rs:53-136) from the host's libm.
//
// Where the reference aborts instead of returning an error (a multi-byte
// character that is not whitespace, an unterminated string literal), this
// reader consumes that character, or the rest of the input.
#include <charconv>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/everett_cuda.h"

namespace ev {
int fail(int code, const char* fmt, ...);
void clear_error();
}  // namespace ev

struct ev_program {
  uint64_t num_qubits = 0, num_classical = 0;
  std::vector<ev_op> ops;
  std::vector<uint64_t> pool;
};

namespace {

constexpr double kPi = 3.141592653589793;         // std::f64::consts::PI
constexpr double kTau = 6.283185307179586;        // std::f64::consts::TAU
constexpr double kFracPi4 = 0.7853981633974483;   // std::f64::consts::FRAC_PI_4
constexpr double kFrac1Sqrt2 = 0.7071067811865476;

struct QasmError {
  uint64_t line, col;
  std::string message;
};

// ---- gate matrices (src/gate.rs:53-136) -------------------------------------

struct M1 {
  double m[8];  // row-major 2x2, interleaved re, im
};

M1 mk(double a, double b, double c, double d, double e, double f, double g, double h) {
  return M1{{a, b, c, d, e, f, g, h}};
}
M1 g_id() { return mk(1, 0, 0, 0, 0, 0, 1, 0); }
M1 g_x() { return mk(0, 0, 1, 0, 1, 0, 0, 0); }
M1 g_y() { return mk(0, 0, 0.0, -1.0, 0.0, 1.0, 0, 0); }
M1 g_z() { return mk(1, 0, 0, 0, 0, 0, -1.0, 0.0); }
M1 g_h() {
  const double s = kFrac1Sqrt2;
  return mk(s, 0.0, s, 0.0, s, 0.0, -s, 0.0);
}
M1 g_s() { return mk(1, 0, 0, 0, 0, 0, 0, 1); }
M1 g_t() { return mk(1, 0, 0, 0, 0, 0, std::cos(kFracPi4), std::sin(kFracPi4)); }
M1 g_rx(double t) {
  const double h = t / 2.0, s = std::sin(h), c = std::cos(h);
  return mk(c, 0.0, 0.0, -s, 0.0, -s, c, 0.0);
}
M1 g_ry(double t) {
  const double h = t / 2.0, s = std::sin(h), c = std::cos(h);
  return mk(c, 0.0, -s, 0.0, s, 0.0, c, 0.0);
}
M1 g_rz(double t) {
  const double a = -t / 2.0, b = t / 2.0;
  return mk(std::cos(a), std::sin(a), 0, 0, 0, 0, std::cos(b), std::sin(b));
}
M1 g_phase(double l) { return mk(1, 0, 0, 0, 0, 0, std::cos(l), std::sin(l)); }

const double kCnot[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                          0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0};
const double kCz[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0,
                        0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, -1.0, 0};
const double kSwap[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0,
                          0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0};

// gates.rs:113-133
M1 lookup_1q(const std::string& name, const std::vector<double>& args) {
  if (args.empty()) {
    if (name == "h") return g_h();
    if (name == "x") return g_x();
    if (name == "y") return g_y();
    if (name == "z") return g_z();
    if (name == "s") return g_s();
    if (name == "t") return g_t();
    if (name == "id") return g_id();
  } else if (args.size() == 1) {
    if (name == "rx") return g_rx(args[0]);
    if (name == "ry") return g_ry(args[0]);
    if (name == "rz") return g_rz(args[0]);
    if (name == "p" || name == "phase") return g_phase(args[0]);
  }
  throw QasmError{0, 0, "unknown single-qubit gate '" + name + "'"};
}

// gates.rs:136-148
const double* lookup_2q(const std::string& name) {
  if (name == "cx" || name == "cnot" || name == "CX") return kCnot;
  if (name == "cz") return kCz;
  if (name == "swap") return kSwap;
  throw QasmError{0, 0, "unknown two-qubit gate '" + name + "'"};
}

// ---- lexer (parse.rs:9-224) --------------------------------------------------

enum Kind {
  T_IDENT, T_INT, T_FLOAT, T_STR, T_OPENQASM, T_INCLUDE, T_QUBIT, T_BIT, T_MEASURE, T_IF, T_GATE,
  T_CTRL, T_PI, T_TAU, T_SEMI, T_LPAREN, T_RPAREN, T_LBRACK, T_RBRACK, T_LBRACE, T_RBRACE,
  T_COMMA, T_EQ, T_EQEQ, T_ARROW, T_SLASH, T_STAR, T_PLUS, T_MINUS, T_AT, T_EOF
};

struct Tok {
  Kind kind = T_EOF;
  std::string text;  // identifier
  uint64_t ival = 0;
  double fval = 0.0;
  uint64_t line = 1, col = 1;
};

// One code point of UTF-8 at p (an invalid byte counts as one code point).
uint32_t decode(const unsigned char* p, size_t avail, size_t* len) {
  const unsigned char b = p[0];
  int n = b < 0x80 ? 1 : (b >> 5) == 6 ? 2 : (b >> 4) == 14 ? 3 : (b >> 3) == 30 ? 4 : 0;
  if (n == 0 || size_t(n) > avail) {
    *len = 1;
    return b;
  }
  uint32_t cp = n == 1 ? b : n == 2 ? (b & 0x1F) : n == 3 ? (b & 0x0F) : (b & 0x07);
  for (int i = 1; i < n; ++i) {
    if ((p[i] >> 6) != 2) {
      *len = 1;
      return b;
    }
    cp = (cp << 6) | (p[i] & 0x3F);
  }
  *len = size_t(n);
  return cp;
}

// char::is_whitespace (Unicode White_Space)
bool is_ws(uint32_t c) {
  return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
         (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F ||
         c == 0x205F || c == 0x3000;
}

bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }
bool is_alpha(unsigned char c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'); }

// str::parse::<f64> of a scanned number, or 0.0 where that parse fails
// (an exponent without digits).
double parse_f64(const std::string& s) {
  const size_t e = s.find_first_of("eE");
  if (e != std::string::npos) {
    size_t i = e + 1;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
    if (i >= s.size()) return 0.0;
  }
  double v = 0.0;
  const auto r = std::from_chars(s.data(), s.data() + s.size(), v);
  // beyond the double range: the correctly rounded inf / subnormal / 0 that
  // Rust's parser gives (the scanned text holds only digits, '.', e, signs)
  if (r.ec == std::errc::result_out_of_range) return std::strtod(s.c_str(), nullptr);
  if (r.ec != std::errc() || r.ptr != s.data() + s.size()) return 0.0;
  return v;
}

class Lexer {
 public:
  Lexer(const char* src, size_t len) : s_(reinterpret_cast<const unsigned char*>(src)), n_(len) {}

  Tok next() {
    skip();
    Tok t;
    t.line = line_;
    t.col = col_;
    if (pos_ >= n_) return t;
    const unsigned char ch = s_[pos_];
    if (ch == '"') {
      size_t j = pos_ + 1;
      while (j < n_ && s_[j] != '"') ++j;
      t.kind = T_STR;
      t.text.assign(reinterpret_cast<const char*>(s_) + pos_ + 1, j - pos_ - 1);
      advance(j < n_ ? j + 1 - pos_ : n_ - pos_);
      return t;
    }
    if (starts("==")) return sym(t, T_EQEQ, 2);
    if (starts("->")) return sym(t, T_ARROW, 2);
    switch (ch) {
      case ';': return sym(t, T_SEMI, 1);
      case '(': return sym(t, T_LPAREN, 1);
      case ')': return sym(t, T_RPAREN, 1);
      case '[': return sym(t, T_LBRACK, 1);
      case ']': return sym(t, T_RBRACK, 1);
      case '{': return sym(t, T_LBRACE, 1);
      case '}': return sym(t, T_RBRACE, 1);
      case ',': return sym(t, T_COMMA, 1);
      case '=': return sym(t, T_EQ, 1);
      case '/': return sym(t, T_SLASH, 1);
      case '*': return sym(t, T_STAR, 1);
      case '+': return sym(t, T_PLUS, 1);
      case '-': return sym(t, T_MINUS, 1);
      case '@': return sym(t, T_AT, 1);
      default: break;
    }
    if (is_digit(ch)) {
      size_t i = pos_;
      while (i < n_ && is_digit(s_[i])) ++i;
      if (i < n_ && s_[i] == '.') {
        ++i;
        while (i < n_ && is_digit(s_[i])) ++i;
      }
      if (i < n_ && (s_[i] == 'e' || s_[i] == 'E')) {
        ++i;
        if (i < n_ && (s_[i] == '+' || s_[i] == '-')) ++i;
        while (i < n_ && is_digit(s_[i])) ++i;
      }
      const std::string num(reinterpret_cast<const char*>(s_) + pos_, i - pos_);
      advance(i - pos_);
      if (num.find_first_of(".eE") != std::string::npos) {
        t.kind = T_FLOAT;
        t.fval = parse_f64(num);
        return t;
      }
      uint64_t v = 0;
      const auto r = std::from_chars(num.data(), num.data() + num.size(), v);
      if (r.ec == std::errc() && r.ptr == num.data() + num.size()) {
        t.kind = T_INT;
        t.ival = v;
      } else {  // beyond usize: the reference re-parses it as f64
        t.kind = T_FLOAT;
        t.fval = parse_f64(num);
      }
      return t;
    }
    if (is_alpha(ch) || ch == '_') {
      size_t i = pos_ + 1;
      while (i < n_ && (is_alpha(s_[i]) || is_digit(s_[i]) || s_[i] == '_')) ++i;
      const std::string w(reinterpret_cast<const char*>(s_) + pos_, i - pos_);
      advance(i - pos_);
      static const struct {
        const char* w;
        Kind k;
      } kw[] = {{"OPENQASM", T_OPENQASM}, {"include", T_INCLUDE}, {"qubit", T_QUBIT},
                {"bit", T_BIT},           {"measure", T_MEASURE}, {"if", T_IF},
                {"gate", T_GATE},         {"ctrl", T_CTRL},       {"pi", T_PI},
                {"tau", T_TAU}};
      for (const auto& e : kw)
        if (w == e.w) {
          t.kind = e.k;
          return t;
        }
      t.kind = T_IDENT;
      t.text = w;
      return t;
    }
    size_t cl = 1;
    decode(s_ + pos_, n_ - pos_, &cl);
    advance(cl);
    t.kind = T_IDENT;
    t.text = "?";
    return t;
  }

 private:
  bool starts(const char* lit) const {
    const size_t l = std::strlen(lit);
    return n_ - pos_ >= l && std::memcmp(s_ + pos_, lit, l) == 0;
  }
  Tok& sym(Tok& t, Kind k, size_t len) {
    advance(len);
    t.kind = k;
    return t;
  }
  void advance(size_t nbytes) {
    const size_t end = pos_ + nbytes;
    while (pos_ < end) {
      size_t cl = 1;
      const uint32_t cp = decode(s_ + pos_, n_ - pos_, &cl);
      if (cp == '\n') {
        ++line_;
        col_ = 1;
      } else {
        ++col_;
      }
      pos_ += cl;
    }
  }
  void skip() {
    for (;;) {
      size_t k = 0;
      while (pos_ + k < n_) {
        size_t cl = 1;
        const uint32_t cp = decode(s_ + pos_ + k, n_ - pos_ - k, &cl);
        if (!is_ws(cp)) break;
        k += cl;
      }
      if (k) {
        advance(k);
        continue;
      }
      if (starts("//")) {
        size_t j = pos_;
        while (j < n_ && s_[j] != '\n') ++j;
        advance(j < n_ ? j + 1 - pos_ : n_ - pos_);
        continue;
      }
      if (starts("/*")) {
        // the terminator is searched from the opening '/', so "/*/" closes
        size_t j = pos_ + 1;
        while (j + 1 < n_ && !(s_[j] == '*' && s_[j + 1] == '/')) ++j;
        advance(j + 1 < n_ ? j + 2 - pos_ : n_ - pos_);
        continue;
      }
      return;
    }
  }

  const unsigned char* s_;
  size_t n_, pos_ = 0;
  uint64_t line_ = 1, col_ = 1;
};

// ---- parser (parse.rs:229-816) -------------------------------------------------

struct Node {
  int kind = 0;  // EV_OP_*
  uint64_t q0 = 0, q1 = 0;
  std::vector<uint64_t> ctrls;
  double m[32] = {};
  std::unique_ptr<Node> inner;
};

class Parser {
 public:
  Parser(const char* src, size_t len) : lex_(src, len) {}

  void program(ev_program* out) {
    uint64_t nq = 0, ncl = 0;
    std::vector<std::unique_ptr<Node>> ops;
    if (peek().kind == T_OPENQASM) {
      consume();
      if (peek().kind == T_INT || peek().kind == T_FLOAT) consume();
      expect_semi();
    }
    if (peek().kind == T_INCLUDE) {
      consume();
      consume();  // the file name
      expect_semi();
    }
    for (;;) {
      const Kind k = peek().kind;
      if (k == T_EOF) break;
      if (k == T_QUBIT || k == T_BIT) {
        consume();
        expect(T_LBRACK, "expected '['");
        const uint64_t n = parse_int();
        expect(T_RBRACK, "expected ']'");
        if (consume().kind != T_IDENT)
          throw err(k == T_QUBIT ? "expected qubit register name"
                                 : "expected classical register name");
        expect_semi();
        (k == T_QUBIT ? nq : ncl) = n;
      } else if (k == T_GATE) {
        consume();
        while (peek().kind != T_LBRACE && peek().kind != T_EOF) consume();
        skip_block();
      } else {
        std::unique_ptr<Node> op = statement();
        if (op) ops.push_back(std::move(op));
      }
    }
    out->num_qubits = nq;
    out->num_classical = ncl;
    for (const auto& op : ops) encode(*op, out);
  }

 private:
  const Tok& peek() {
    if (!has_peek_) {
      peek_ = lex_.next();
      has_peek_ = true;
    }
    return peek_;
  }
  Tok consume() {
    if (has_peek_) {
      has_peek_ = false;
      return std::move(peek_);
    }
    return lex_.next();
  }
  QasmError err(const std::string& msg) {
    const Tok& t = peek();
    return QasmError{t.line, t.col, msg};
  }
  void expect(Kind k, const char* msg) {
    if (peek().kind != k) throw err(msg);
    consume();
  }
  void expect_semi() { expect(T_SEMI, "expected ';'"); }
  uint64_t parse_int() {
    const Tok t = consume();
    if (t.kind != T_INT) throw err("expected integer");
    return t.ival;
  }
  uint64_t index() {
    expect(T_LBRACK, "expected '['");
    const uint64_t i = parse_int();
    expect(T_RBRACK, "expected ']'");
    return i;
  }
  uint64_t reg_index(const char* what) {
    if (peek().kind != T_IDENT) throw err(std::string("expected ") + what + " register name");
    consume();
    return index();
  }
  void skip_block() {
    if (consume().kind != T_LBRACE) throw err("expected '{' for gate body");
    uint64_t depth = 1;
    for (;;) {
      const Kind k = consume().kind;
      if (k == T_LBRACE) {
        ++depth;
      } else if (k == T_RBRACE) {
        if (--depth == 0) return;
      } else if (k == T_EOF) {
        throw err("unexpected EOF in gate body");
      }
    }
  }

  std::unique_ptr<Node> statement() {
    const Kind k = peek().kind;
    if (k == T_SEMI) {
      consume();
      return nullptr;
    }
    if (k == T_MEASURE) {
      consume();
      auto n = std::make_unique<Node>();
      n->kind = EV_OP_MEASURE;
      n->q0 = reg_index("qubit");
      const Kind k2 = peek().kind;
      if (k2 == T_ARROW) {
        consume();
        n->q1 = reg_index("classical");
        expect_semi();
        return n;
      }
      if (k2 == T_SEMI) {
        consume();
        throw QasmError{0, 0, "bare 'measure' without destination is not supported"};
      }
      throw err("expected '->' or ';' after measure operand");
    }
    if (k == T_IF) return parse_if();
    if (k == T_CTRL) return ctrl_call();
    if (k == T_IDENT) {
      const std::string name = peek().text;
      if (name == "reset" || name == "barrier") {
        for (;;) {
          const Kind kk = consume().kind;
          if (kk == T_SEMI || kk == T_EOF) break;
        }
        return nullptr;
      }
      consume();
      const Kind k2 = peek().kind;
      if (k2 == T_LBRACK) {
        consume();
        const uint64_t idx = parse_int();
        expect(T_RBRACK, "expected ']'");
        if (peek().kind != T_EQ) throw err("unexpected token after register index");
        consume();
        if (peek().kind != T_MEASURE) throw err("expected 'measure' after '='");
        consume();
        auto n = std::make_unique<Node>();
        n->kind = EV_OP_MEASURE;
        n->q0 = reg_index("qubit");
        n->q1 = idx;
        expect_semi();
        return n;
      }
      if (k2 == T_LPAREN || k2 == T_IDENT || k2 == T_SEMI || k2 == T_COMMA)
        return call_after_name(name);
      throw err("unexpected token in statement");
    }
    consume();
    return nullptr;
  }

  std::unique_ptr<Node> parse_if() {
    consume();
    if (consume().kind != T_LPAREN) throw err("expected '(' after 'if'");
    if (consume().kind != T_IDENT) throw err("expected classical register in if condition");
    expect(T_LBRACK, "expected '['");
    const uint64_t bit = parse_int();
    expect(T_RBRACK, "expected ']'");
    if (consume().kind != T_EQEQ) throw err("expected '==' in if condition");
    const Tok one = consume();
    if (!(one.kind == T_INT && one.ival == 1))
      throw QasmError{0, 0, "only 'if (c[i] == 1)' is supported"};
    if (consume().kind != T_RPAREN) throw err("expected ')' to close if condition");
    std::unique_ptr<Node> inner = statement();
    if (!inner) throw err("expected statement in if body");
    auto n = std::make_unique<Node>();
    n->kind = EV_OP_IF;
    n->q0 = bit;
    n->inner = std::move(inner);
    return n;
  }

  // A gate-table error takes the position of the token after the statement.
  template <typename F>
  auto with_pos(F f) -> decltype(f()) {
    try {
      return f();
    } catch (QasmError& e) {
      const Tok& t = peek();
      e.line = t.line;
      e.col = t.col;
      throw;
    }
  }

  std::unique_ptr<Node> ctrl_call() {
    consume();
    uint64_t nctrl = 1;
    if (peek().kind == T_LPAREN) {
      consume();
      nctrl = parse_int();
      if (consume().kind != T_RPAREN) throw err("expected ')'");
    }
    if (consume().kind != T_AT) throw err("expected '@' after ctrl");
    const Tok name = consume();
    if (name.kind != T_IDENT) throw err("expected gate name after 'ctrl @'");
    const std::vector<double> args = arg_list();
    const std::vector<uint64_t> opnds = operand_list();
    expect_semi();
    if (uint64_t(opnds.size()) < nctrl + 1 || nctrl + 1 == 0)
      throw err("not enough operands for ctrl gate");
    const M1 g = with_pos([&] { return lookup_1q(name.text, args); });
    auto n = std::make_unique<Node>();
    n->kind = EV_OP_CONTROLLED;
    n->ctrls.assign(opnds.begin(), opnds.begin() + long(nctrl));
    n->q0 = opnds[nctrl];
    std::memcpy(n->m, g.m, sizeof(g.m));
    return n;
  }

  std::unique_ptr<Node> call_after_name(const std::string& name) {
    const std::vector<double> args = arg_list();
    const std::vector<uint64_t> opnds = operand_list();
    expect_semi();
    auto n = std::make_unique<Node>();
    if (opnds.size() == 1) {
      const M1 g = with_pos([&] { return lookup_1q(name, args); });
      n->kind = EV_OP_APPLY1;
      n->q0 = opnds[0];
      std::memcpy(n->m, g.m, sizeof(g.m));
      return n;
    }
    if (opnds.size() == 2 && args.empty()) {
      const double* m = with_pos([&] { return lookup_2q(name); });
      n->kind = EV_OP_APPLY2;
      n->q0 = opnds[0];
      n->q1 = opnds[1];
      std::memcpy(n->m, m, 32 * sizeof(double));
      return n;
    }
    throw err("unexpected gate arity");
  }

  std::vector<double> arg_list() {
    std::vector<double> a;
    if (peek().kind != T_LPAREN) return a;
    consume();
    for (;;) {
      const Kind k = peek().kind;
      if (k == T_RPAREN) {
        consume();
        return a;
      }
      if (k == T_COMMA)
        consume();
      else
        a.push_back(expr());
    }
  }

  std::vector<uint64_t> operand_list() {
    std::vector<uint64_t> out;
    for (;;) {
      const Kind k = peek().kind;
      if (k == T_IDENT) {
        consume();
        out.push_back(index());
      } else if (k == T_COMMA) {
        consume();
      } else {
        return out;
      }
    }
  }

  double expr() {
    double lhs = mul();
    for (;;) {
      const Kind k = peek().kind;
      if (k == T_PLUS) {
        consume();
        lhs = lhs + mul();
      } else if (k == T_MINUS) {
        consume();
        lhs = lhs - mul();
      } else {
        return lhs;
      }
    }
  }
  double mul() {
    double lhs = unary();
    for (;;) {
      const Kind k = peek().kind;
      if (k == T_STAR) {
        consume();
        lhs = lhs * unary();
      } else if (k == T_SLASH) {
        consume();
        const double rhs = unary();
        if (rhs == 0.0) throw err("division by zero in angle expression");
        lhs = lhs / rhs;
      } else {
        return lhs;
      }
    }
  }
  double unary() {
    const Kind k = peek().kind;
    if (k == T_MINUS) {
      consume();
      return -primary();
    }
    if (k == T_PLUS) consume();
    return primary();
  }
  double primary() {
    const Tok t = consume();
    switch (t.kind) {
      case T_FLOAT: return t.fval;
      case T_INT: return double(t.ival);
      case T_PI: return kPi;
      case T_TAU: return kTau;
      case T_LPAREN: {
        const double v = expr();
        if (consume().kind != T_RPAREN) throw err("expected ')'");
        return v;
      }
      default: throw err("expected numeric expression");
    }
  }

  static void encode(const Node& n, ev_program* out) {
    ev_op op;
    std::memset(&op, 0, sizeof(op));
    op.kind = uint32_t(n.kind);
    op.q0 = n.q0;
    op.q1 = n.q1;
    if (n.kind == EV_OP_APPLY2)
      std::memcpy(op.m, n.m, 32 * sizeof(double));
    else if (n.kind == EV_OP_APPLY1 || n.kind == EV_OP_CONTROLLED)
      std::memcpy(op.m, n.m, 8 * sizeof(double));
    if (n.kind == EV_OP_CONTROLLED) {
      op.nctrl = uint32_t(n.ctrls.size());
      op.ctrl_off = out->pool.size();
      out->pool.insert(out->pool.end(), n.ctrls.begin(), n.ctrls.end());
    }
    out->ops.push_back(op);
    if (n.kind == EV_OP_IF) encode(*n.inner, out);
  }

  Lexer lex_;
  Tok peek_;
  bool has_peek_ = false;
};

// ---- emitter (emit.rs:17-81, gates.rs:28-111) -------------------------------------

bool eq_m(const double* a, const M1& b) {
  for (int i = 0; i < 8; ++i)
    if (!(a[i] == b.m[i])) return false;
  return true;
}
bool close_m(const double* a, const M1& b) {
  for (int k = 0; k < 4; ++k)
    if (!(std::hypot(a[2 * k] - b.m[2 * k], a[2 * k + 1] - b.m[2 * k + 1]) < 1e-12)) return false;
  return true;
}

std::string angle(double v) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "(%.17f)", v);
  return buf;
}

std::string gate_name_1q(const double* m) {
  if (eq_m(m, g_x())) return "x";
  if (eq_m(m, g_y())) return "y";
  if (eq_m(m, g_z())) return "z";
  if (eq_m(m, g_h())) return "h";
  if (eq_m(m, g_s())) return "s";
  if (eq_m(m, g_t())) return "t";
  if (eq_m(m, g_id())) return "id";
  // m[k] = (m[2k], m[2k+1])
  if (m[1] == 0.0 && m[2] == 0.0 && m[4] == 0.0 && m[7] == 0.0 && std::fabs(m[0] - m[6]) < 1e-15) {
    const double theta = 2.0 * std::atan2(-m[5], m[0]);
    if (close_m(m, g_rx(theta))) return "rx" + angle(theta);
  }
  if (m[1] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[7] == 0.0 && std::fabs(m[0] - m[6]) < 1e-15 &&
      std::fabs(m[2] + m[4]) < 1e-15) {
    const double theta = 2.0 * std::atan2(m[4], m[0]);
    if (close_m(m, g_ry(theta))) return "ry" + angle(theta);
  }
  if (m[2] == 0.0 && m[3] == 0.0 && m[4] == 0.0 && m[5] == 0.0) {
    const double theta = -2.0 * std::atan2(m[1], m[0]);
    if (close_m(m, g_rz(theta))) return "rz" + angle(theta);
    const double lambda = std::atan2(m[7], m[6]);
    if (close_m(m, g_phase(lambda))) return "p" + angle(lambda);
  }
  throw QasmError{0, 0, "gate has no OpenQASM 3 name; use a named gate constructor"};
}

std::string gate_name_2q(const double* m) {
  auto same = [&](const double* k) {
    for (int i = 0; i < 32; ++i)
      if (!(m[i] == k[i])) return false;
    return true;
  };
  if (same(kCnot)) return "cx";
  if (same(kCz)) return "cz";
  if (same(kSwap)) return "swap";
  throw QasmError{0, 0, "gate has no OpenQASM 3 name; use a named gate constructor"};
}

std::string q(uint64_t i) { return "q[" + std::to_string(i) + "]"; }

void emit_op(const ev_circuit* c, uint64_t* pos, int depth, std::string* out) {
  if (*pos >= c->nops) throw QasmError{0, 0, "op list ends inside an IfClassic record"};
  const ev_op& op = c->ops[*pos];
  *pos += 1;
  switch (op.kind) {
    case EV_OP_APPLY1:
      *out += gate_name_1q(op.m) + " " + q(op.q0) + ";";
      return;
    case EV_OP_APPLY2:
      *out += gate_name_2q(op.m) + " " + q(op.q0) + ", " + q(op.q1) + ";";
      return;
    case EV_OP_CONTROLLED: {
      const std::string g = gate_name_1q(op.m);
      *out += op.nctrl == 1 ? std::string("ctrl @ ") : "ctrl(" + std::to_string(op.nctrl) + ") @ ";
      *out += g + " ";
      for (uint32_t j = 0; j < op.nctrl; ++j) *out += q(c->ctrl_pool[op.ctrl_off + j]) + ", ";
      *out += q(op.q0) + ";";
      return;
    }
    case EV_OP_MEASURE:
      *out += "c[" + std::to_string(op.q1) + "] = measure " + q(op.q0) + ";";
      return;
    case EV_OP_IF:
      if (depth > 0)
        throw QasmError{0, 0, "nested IfClassic is not supported in OpenQASM 3 emit"};
      *out += "if (c[" + std::to_string(op.q0) + "] == 1) ";
      emit_op(c, pos, depth + 1, out);
      return;
    default:
      throw QasmError{0, 0, "unknown op kind " + std::to_string(op.kind)};
  }
}

int qasm_fail(const QasmError& e) {
  return ev::fail(EV_ERR_QASM, "OpenQASM 3 error at %llu:%llu: %s", (unsigned long long)e.line,
                  (unsigned long long)e.col, e.message.c_str());
}

}  // namespace

extern "C" int ev_qasm_parse(const char* src, uint64_t len, ev_program** out, uint64_t* err_line,
                             uint64_t* err_col) {
  ev::clear_error();
  if (!out || (len && !src)) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_qasm_parse: null argument");
  *out = nullptr;
  std::unique_ptr<ev_program> p(new ev_program());
  try {
    Parser(src ? src : "", size_t(len)).program(p.get());
  } catch (const QasmError& e) {
    if (err_line) *err_line = e.line;
    if (err_col) *err_col = e.col;
    return qasm_fail(e);
  } catch (const std::bad_alloc&) {
    return ev::fail(EV_ERR_OOM, "ev_qasm_parse: out of host memory");
  }
  *out = p.release();
  return EV_OK;
}

extern "C" int ev_program_circuit(const ev_program* p, ev_circuit* out) {
  ev::clear_error();
  if (!p || !out) return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_program_circuit: null argument");
  out->num_qubits = p->num_qubits;
  out->num_classical = p->num_classical;
  out->ops = p->ops.empty() ? nullptr : p->ops.data();
  out->nops = p->ops.size();
  out->ctrl_pool = p->pool.empty() ? nullptr : p->pool.data();
  out->pool_len = p->pool.size();
  return EV_OK;
}

extern "C" int ev_program_free(ev_program* p) {
  ev::clear_error();
  delete p;
  return EV_OK;
}

extern "C" int ev_qasm_emit(const ev_circuit* c, char* buf, uint64_t cap, uint64_t* len) {
  ev::clear_error();
  if (!c || !len || (c->nops && !c->ops))
    return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_qasm_emit: null argument");
  std::string s;
  try {
    s = "OPENQASM 3.0;\ninclude \"stdgates.inc\";\n";
    if (c->num_qubits > 0) s += "qubit[" + std::to_string(c->num_qubits) + "] q;\n";
    if (c->num_classical > 0) s += "bit[" + std::to_string(c->num_classical) + "] c;\n";
    s += "\n";
    uint64_t pos = 0;
    while (pos < c->nops) {
      emit_op(c, &pos, 0, &s);
      s += "\n";
    }
  } catch (const QasmError& e) {
    return qasm_fail(e);
  } catch (const std::bad_alloc&) {
    return ev::fail(EV_ERR_OOM, "ev_qasm_emit: out of host memory");
  }
  *len = s.size();
  if (!buf) return EV_OK;
  if (cap < s.size() + 1)
    return ev::fail(EV_ERR_INVALID_ARGUMENT, "ev_qasm_emit: buffer of %llu bytes, %llu needed",
                    (unsigned long long)cap, (unsigned long long)(s.size() + 1));
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return EV_OK;
}

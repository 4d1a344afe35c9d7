// IR parsing and CUDA C generation for the fused kernels.
//
// The generated kernels compute, per output point, exactly the statement list
// the reference's OpenCL kernel builder emits for the same tree
// (OpenCLKernelBuilder/src/main/scala/com/thoughtworks/compute/
// OpenCLKernelBuilder.scala): one `const float` per operator node (:245-326,
// :516-571), view indices as `(int)(sum of gid * coefficient + constant)` with
// the coefficients printed by DecimalFormat (:14-32, :348-386), and an
// out-of-range view index reading the parameter's padding (:387-411).  Around
// that statement list sit the sm_103a skeletons: a grid-stride elementwise
// loop (with a float4 variant when every input is read contiguously) and a
// compensated full sum with a single-pass grid reduction.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <sstream>
#include <initializer_list>
#include <utility>

#include "internal.h"

namespace cc {

// ---------------------------------------------------------------- parsing

namespace {

struct Tok {
  const char *p, *end;
  bool eol() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    return p >= end || *p == '\n';
  }
  std::string word() {
    if (eol()) fail(CC_ERR_INVALID_PROGRAM, "IR: unexpected end of line");
    const char *s = p;
    while (p < end && *p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') ++p;
    return std::string(s, p);
  }
  int64_t integer() {
    std::string w = word();
    char *e = nullptr;
    long long v = strtoll(w.c_str(), &e, 10);
    if (*e) fail(CC_ERR_INVALID_PROGRAM, "IR: bad integer '" + w + "'");
    return v;
  }
  double real() {
    std::string w = word();
    char *e = nullptr;
    double v = strtod(w.c_str(), &e);
    if (*e) fail(CC_ERR_INVALID_PROGRAM, "IR: bad number '" + w + "'");
    return v;
  }
  uint32_t hex32() {
    std::string w = word();
    char *e = nullptr;
    unsigned long v = strtoul(w.c_str(), &e, 16);
    if (*e || w.size() != 8) fail(CC_ERR_INVALID_PROGRAM, "IR: bad float bits '" + w + "'");
    return (uint32_t)v;
  }
  void next_line() {
    if (!eol()) fail(CC_ERR_INVALID_PROGRAM, "IR: trailing tokens");
    if (p < end) ++p;
  }
};

const char *kUnNames[] = {"neg", "exp", "log", "tanh", "abs", "sqrt"};
const char *kBinNames[] = {"add", "sub", "mul", "div", "mod", "min", "max"};

}  // namespace

Ir parse_ir(const char *text, size_t len) {
  Ir ir;
  Tok t{text, text + len};
  if (t.word() != "ccir" || t.integer() != 1) fail(CC_ERR_INVALID_PROGRAM, "IR: missing 'ccir 1' header");
  std::string kind = t.word();
  if (kind == "ew") ir.kind = ProgramKind::Elementwise;
  else if (kind == "sum") ir.kind = ProgramKind::Sum;
  else fail(CC_ERR_INVALID_PROGRAM, "IR: unknown program kind '" + kind + "'");
  t.next_line();
  if (t.word() != "o") fail(CC_ERR_INVALID_PROGRAM, "IR: missing output shape");
  int64_t rank = t.integer();
  if (rank < 0 || rank > 16) fail(CC_ERR_INVALID_PROGRAM, "IR: output rank out of range");
  for (int64_t i = 0; i < rank; ++i) {
    int64_t d = t.integer();
    if (d < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: negative dimension");
    ir.out_shape.push_back(d);
  }
  t.next_line();
  auto node_ref = [&](int64_t v) -> int {
    if (v < 0 || v >= (int64_t)ir.nodes.size()) fail(CC_ERR_INVALID_PROGRAM, "IR: operand refers forward or out of range");
    return (int)v;
  };
  while (t.p < t.end) {
    if (t.eol()) { t.next_line(); continue; }
    std::string tag = t.word();
    if (tag == "r") {
      ir.root = node_ref(t.integer());
      t.next_line();
      while (t.p < t.end) {
        if (!t.eol()) fail(CC_ERR_INVALID_PROGRAM, "IR: content after root");
        t.next_line();
      }
      break;
    }
    IrNode n;
    if (tag == "p") {
      n.kind = NodeKind::Param;
      int64_t r = t.integer();
      if (r < 0 || r > 16) fail(CC_ERR_INVALID_PROGRAM, "IR: parameter rank out of range");
      for (int64_t i = 0; i < r; ++i) {
        int64_t d = t.integer();
        if (d < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: negative dimension");
        n.dims.push_back(d);
      }
      n.bits = t.hex32();
      n.param_index = ir.n_params++;
      ir.param_nodes.push_back((int)ir.nodes.size());
    } else if (tag == "l") {
      n.kind = NodeKind::Literal;
      n.bits = t.hex32();
    } else if (tag == "x") {
      n.kind = NodeKind::Extract;
      n.a = node_ref(t.integer());
      if (ir.nodes[n.a].kind != NodeKind::Param) fail(CC_ERR_INVALID_PROGRAM, "IR: extract of a non-parameter");
      n.cols = (int)t.integer();
      size_t rows = ir.nodes[n.a].dims.size();
      if (n.cols < 1 || n.cols > 17) fail(CC_ERR_INVALID_PROGRAM, "IR: bad matrix columns");
      for (size_t i = 0; i < rows * (size_t)n.cols; ++i) n.m.push_back(t.real());
    } else if (tag == "v") {
      n.kind = NodeKind::View;
      n.a = node_ref(t.integer());
      int64_t r = t.integer();
      if (r < 0 || r > 16) fail(CC_ERR_INVALID_PROGRAM, "IR: view rank out of range");
      for (int64_t i = 0; i < r; ++i) {
        int64_t d = t.integer();
        if (d < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: negative dimension");
        n.dims.push_back(d);
      }
      n.bits = t.hex32();
      n.cols = (int)t.integer();
      if (n.cols < 1 || n.cols > 17) fail(CC_ERR_INVALID_PROGRAM, "IR: bad matrix columns");
      for (size_t i = 0; i < (size_t)r * (size_t)n.cols; ++i) n.m.push_back(t.real());
    } else if (tag == "u") {
      n.kind = NodeKind::Unary;
      std::string op = t.word();
      int k = -1;
      for (int i = 0; i < 6; ++i) if (op == kUnNames[i]) k = i;
      if (k < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: unknown unary operator '" + op + "'");
      n.op = (uint8_t)k;
      n.a = node_ref(t.integer());
    } else if (tag == "b") {
      n.kind = NodeKind::Binary;
      std::string op = t.word();
      int k = -1;
      for (int i = 0; i < 7; ++i) if (op == kBinNames[i]) k = i;
      if (k < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: unknown binary operator '" + op + "'");
      n.op = (uint8_t)k;
      n.a = node_ref(t.integer());
      n.b = node_ref(t.integer());
    } else if (tag == "t") {
      n.kind = NodeKind::Tuple;
      int64_t cnt = t.integer();
      if (cnt < 1 || cnt > 4096) fail(CC_ERR_INVALID_PROGRAM, "IR: bad tuple length");
      for (int64_t i = 0; i < cnt; ++i) n.elems.push_back(node_ref(t.integer()));
    } else {
      fail(CC_ERR_INVALID_PROGRAM, "IR: unknown line tag '" + tag + "'");
    }
    t.next_line();
    ir.nodes.push_back(std::move(n));
  }
  if (ir.root < 0) fail(CC_ERR_INVALID_PROGRAM, "IR: missing root");
  for (size_t i = 0; i < ir.nodes.size(); ++i) {
    if (ir.nodes[i].kind == NodeKind::Tuple && (int)i != ir.root)
      fail(CC_ERR_INVALID_PROGRAM, "IR: a tuple may only be the root");
  }
  if (ir.kind == ProgramKind::Sum && ir.nodes[ir.root].kind == NodeKind::Tuple)
    fail(CC_ERR_INVALID_PROGRAM, "IR: the sum of a tuple-valued tree is not defined");
  return ir;
}

// ---------------------------------------------------------------- literals

std::string decimal_format3(double v) {
  // Exact decimal expansion of the double, then HALF_EVEN rounding at the third
  // fraction digit (java.text.DecimalFormat's default pattern "#,##0.###" with
  // grouping off).
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "\xE2\x88\x9E" : "-\xE2\x88\x9E";
  bool neg = std::signbit(v);
  double a = std::fabs(v);
  static thread_local char buf[1600];
  snprintf(buf, sizeof buf, "%.1100f", a);
  std::string s(buf);
  size_t dot = s.find('.');
  std::string ip = s.substr(0, dot);
  std::string fp = s.substr(dot + 1);
  std::string keep = fp.substr(0, 3);
  std::string rest = fp.substr(3);
  int cmp;  // rest vs one half
  if (rest.empty() || rest[0] < '5') {
    cmp = -1;
  } else if (rest[0] > '5') {
    cmp = 1;
  } else {
    cmp = (rest.find_first_not_of('0', 1) == std::string::npos) ? 0 : 1;
  }
  std::string digits = ip + keep;
  bool up = cmp > 0 || (cmp == 0 && ((digits.back() - '0') % 2 == 1));
  if (up) {
    int i = (int)digits.size() - 1;
    while (i >= 0) {
      if (digits[i] == '9') { digits[i] = '0'; --i; }
      else { digits[i]++; break; }
    }
    if (i < 0) digits.insert(digits.begin(), '1');
  }
  std::string ipart = digits.substr(0, digits.size() - 3);
  std::string fpart = digits.substr(digits.size() - 3);
  size_t nz = ipart.find_first_not_of('0');
  ipart = nz == std::string::npos ? "0" : ipart.substr(nz);
  while (!fpart.empty() && fpart.back() == '0') fpart.pop_back();
  std::string out = (neg ? "-" : "") + ipart;
  if (!fpart.empty()) out += "." + fpart;
  return out;
}

// ---------------------------------------------------------------- generation

namespace {

}  // namespace
// device_common.cuh, embedded at build time as a string literal.
extern const char *kPrelude;
const char *kPrelude =
#include "device_common.inc"
    ;
namespace {

std::string lit_code(uint32_t bits) {
  char b[48];
  snprintf(b, sizeof b, "__int_as_float(0x%08x)", bits);
  return b;
}

struct Frame {
  int id;
  std::vector<std::string> gid;   // index variable names
  std::vector<int64_t> shape;
  std::vector<int64_t> goff = {};  // constant added to each index variable (empty: none)
  // Index variables whose value is a compile-time integer (a view row with no
  // coordinate term): gknown[x] != 0 means gid[x] == gval[x] (empty: none).
  std::vector<uint8_t> gknown = {};
  std::vector<int64_t> gval = {};
};

// One generated statement.  Index statements are integer view arithmetic (they
// depend only on coordinates), loads read a buffer, computes are float ops.
enum class Cat : uint8_t { Index, Prefetch, Load, Compute };
struct Stmt {
  Cat cat;
  std::string text;
  // A load staged through the shared-memory ring: its order among ring loads,
  // the variable it defines, its address, its bounds condition ("" = none)
  // and the input it reads (an in-bounds address when the condition fails).
  int ring = -1;
  std::string var, ptr, ok, base;
  // A load at an index that depends on no output coordinate: its parameter,
  // offset expression and padding, so it can be redirected to a shared copy.
  int uparam = -1;
  std::string uoff;
  uint32_t ubits = 0;
  // Emission order of loads and arithmetic (stable; creation order unless
  // statements are merged across points, see Generator::set_point).
  int64_t key = 0;
  // A scalar predicated load (var, ptr, ok, padding ubits) that emit() may put
  // in one inline-PTX block with its neighbours of the same condition.
  bool batchable = false;
};

}  // namespace

thread_local bool g_codegen_fma = false;

namespace {

class Generator {
 public:
  Generator(const Ir &ir, bool contiguous_mode, bool asm_loads = false, int64_t prefetch_min_bytes = -1,
            bool shared_transcendentals = false)
      : ir_(ir), contig_(contiguous_mode), asm_loads_(asm_loads), prefetch_min_bytes_(prefetch_min_bytes),
        shared_transcendentals_(shared_transcendentals), fma_(g_codegen_fma) {}

  // Returns the name of the variable holding node `n` evaluated in frame `f`;
  // the statements computing it are appended to the statement list.
  std::string gen(int n, const Frame &f) {
    auto key = std::make_pair(n, f.id);
    auto it = memo_.find(key);
    if (it != memo_.end()) return it->second;
    const IrNode &node = ir_.nodes[n];
    std::string v;
    switch (node.kind) {
      case NodeKind::Literal:
        v = fresh();
        if (reuse("K " + lit_code(node.bits), v)) break;
        add(Cat::Compute, "const " + ty() + " " + v + " = " + lit_code(node.bits) + ";");
        break;
      case NodeKind::Unary: {
        std::string a = gen(node.a, f);
        v = fresh();
        if (reuse("U " + std::to_string(node.op) + " " + a, v)) break;
        static const char *fn[] = {"-", "expf", "logf", "tanhf", "fabsf", "sqrtf"};
        static const char *shared_fn[] = {"-", "cc_expf", "cc_logf", "cc_tanhf", "fabsf", "sqrtf"};
        static const char *lane_fn[] = {"-", "cc_exp", "cc_log", "cc_tanh", "cc_abs", "cc_sqrt"};
        if (node.op == (uint8_t)UnOp::Neg)
          add(Cat::Compute, "const " + ty() + " " + v + " = -" + a + ";");
        else
          add(Cat::Compute, "const " + ty() + " " + v + " = " +
                                (lanes_ ? lane_fn : shared_transcendentals_ ? shared_fn : fn)[node.op] + "(" + a + ");");
        break;
      }
      case NodeKind::Binary: {
        if (fma_ && (node.op == (uint8_t)BinOp::Add || node.op == (uint8_t)BinOp::Sub)) {
          // FMA contraction: a product operand of + or - fuses into one fmaf
          // (the left one when both are products), rounded once:
          //   p*q + c, c + p*q -> fmaf(p, q, c);  p*q - c -> fmaf(p, q, -c);  c - p*q -> fmaf(-p, q, c)
          const IrNode &na = ir_.nodes[node.a], &nb = ir_.nodes[node.b];
          const bool a_mul = na.kind == NodeKind::Binary && na.op == (uint8_t)BinOp::Mul;
          const bool b_mul = nb.kind == NodeKind::Binary && nb.op == (uint8_t)BinOp::Mul;
          if (a_mul || b_mul) {
            const IrNode &m = a_mul ? na : nb;
            std::string p = gen(m.a, f);
            std::string q = gen(m.b, f);
            std::string c = gen(a_mul ? node.b : node.a, f);
            v = fresh();
            std::string e;
            const std::string fma = lanes_ ? "cc_fma(" : "__fmaf_rn(";
            if (node.op == (uint8_t)BinOp::Add)
              e = fma + p + ", " + q + ", " + c + ")";
            else if (a_mul)
              e = fma + p + ", " + q + ", -" + c + ")";
            else
              e = fma + "-" + p + ", " + q + ", " + c + ")";
            if (reuse("B " + e, v)) break;
            add(Cat::Compute, "const " + ty() + " " + v + " = " + e + ";");
            break;
          }
        }
        std::string a = gen(node.a, f);
        std::string b = gen(node.b, f);
        v = fresh();
        std::string e;
        switch ((BinOp)node.op) {
          case BinOp::Add: e = a + " + " + b; break;
          case BinOp::Sub: e = a + " - " + b; break;
          case BinOp::Mul: e = a + " * " + b; break;
          case BinOp::Div: e = a + " / " + b; break;
          case BinOp::Mod: e = (lanes_ ? "cc_mod(" : "fmodf(") + a + ", " + b + ")"; break;
          case BinOp::Min: e = (lanes_ ? "cc_min(" : "fminf(") + a + ", " + b + ")"; break;
          case BinOp::Max: e = (lanes_ ? "cc_max(" : "fmaxf(") + a + ", " + b + ")"; break;
        }
        if (reuse("B " + e, v)) break;
        add(Cat::Compute, "const " + ty() + " " + v + " = " + e + ";");
        break;
      }
      case NodeKind::Extract: {
        const IrNode &p = ir_.nodes[node.a];
        if (node.cols != (int)f.shape.size() + 1)
          fail(CC_ERR_INVALID_PROGRAM, "IR: view matrix columns do not match the frame rank");
        v = fresh();
        if (contig_) {
          add(Cat::Compute, "const " + ty() + " " + v + " = a" + std::to_string(p.param_index) + ";");
          break;
        }
        std::vector<std::string> idx, row_ok;
        std::vector<std::pair<bool, int64_t>> rc;
        std::string ok = index_rows(node, p.dims, f, idx, &row_ok, &rc);
        std::string off = offset_expr(p.dims, idx);
        std::string ptr = "in" + std::to_string(p.param_index) + (p.dims.empty() ? "" : " + " + off);
        // A load whose address depends on no output coordinate reads the same
        // word in every thread (an L1 hit after the first): it is emitted where
        // it is used, so the lookahead window holds only loads that go to DRAM.
        bool uniform = true;
        for (const std::string &i : idx)
          if (!uniform_.count(i)) uniform = false;
        const Cat load_cat = uniform ? Cat::Compute : Cat::Load;
        if (!uniform) varying_params_.insert(p.param_index);
        if (vec_loads_ && asm_loads_ && merge_ &&
            vector_load(p, idx, row_ok, rc, !uniform || !staged_.count(p.param_index), !uniform, v))
          break;
        if (reuse("L " + ptr + " " + ok + " " + lit_code(p.bits), v)) break;
        if (ring_ > 0 && !uniform && asm_loads_ && (ok.empty() || p.bits == 0)) {
          // zero padding is the copy's zero fill
          Stmt st{Cat::Load, std::string()};
          st.ring = ring_loads_++;
          st.var = v;
          st.ptr = ptr;
          st.ok = ok;
          st.base = "in" + std::to_string(p.param_index);
          push(std::move(st));
          break;
        }
        if (prefetch_min_bytes_ >= 0) {
          int64_t bytes = 4;
          for (int64_t d : p.dims) bytes *= d;
          if (bytes >= prefetch_min_bytes_)
            add(Cat::Prefetch, "cc_prefetch(" + ptr + ", " + (ok.empty() ? std::string("1") : "(" + ok + ")") + ");");
        }
        if (asm_loads_) {
          // A predicated non-coherent load in volatile inline PTX: the compiler
          // keeps these in the order emit() places them, so the lookahead holds.
          add(load_cat, "float " + v + " = " + lit_code(p.bits) + "; cc_ld(" + v + ", " + ptr + ", " +
                            (ok.empty() ? std::string("1") : "(" + ok + ")") + ");");
          if (!uniform && batch_loads_) {
            Stmt &st = stmts_.back();
            st.batchable = true;
            st.var = v;
            st.ptr = ptr;
            st.ok = ok;
            st.ubits = p.bits;
          }
        } else if (ok.empty()) {
          add(load_cat, "const float " + v + " = __ldg(" + ptr + ");");
        } else {
          add(load_cat, "const float " + v + " = (" + ok + ") ? __ldg(" + ptr + ") : " + lit_code(p.bits) + ";");
        }
        if (uniform) {
          Stmt &st = stmts_.back();
          st.uparam = p.param_index;
          st.uoff = p.dims.empty() ? std::string("0") : off;
          st.ok = ok;
          st.var = v;
          st.ubits = p.bits;
        }
        break;
      }
      case NodeKind::View: {
        // An inline tensor evaluated at view coordinates.  Its expression is
        // evaluated unconditionally and the padding selected afterwards: every
        // load inside carries its own bounds check, so coordinates outside the
        // view cannot read outside a buffer, and the code stays straight-line,
        // so the loads of many views can be scheduled ahead together.
        if (node.cols != (int)f.shape.size() + 1)
          fail(CC_ERR_INVALID_PROGRAM, "IR: view matrix columns do not match the frame rank");
        v = fresh();
        std::vector<std::string> idx;
        std::vector<std::pair<bool, int64_t>> rc;
        std::string ok = index_rows(node, node.dims, f, idx, nullptr, &rc);
        Frame inner{next_frame_++, idx, node.dims};
        for (auto &k : rc) {
          inner.gknown.push_back(k.first ? 1 : 0);
          inner.gval.push_back(k.second);
        }
        std::string sub = gen(node.a, inner);
        if (reuse("V " + ok + " " + sub + " " + lit_code(node.bits), v)) break;
        if (!ok.empty())
          add(Cat::Compute, "const float " + v + " = (" + ok + ") ? " + sub + " : " + lit_code(node.bits) + ";");
        else
          add(Cat::Compute, "const float " + v + " = " + sub + ";");
        break;
      }
      case NodeKind::Param:
        fail(CC_ERR_INVALID_PROGRAM, "IR: a parameter is used as a value without Extract");
      case NodeKind::Tuple:
        fail(CC_ERR_INVALID_PROGRAM, "IR: nested tuple");
    }
    memo_[key] = v;
    return v;
  }

  // Writes the statements in an order the hardware likes: all index arithmetic
  // first, then each load `lookahead` loads ahead of the arithmetic that uses
  // it, so a thread keeps that many independent loads in flight while the
  // float statements still execute in the tree's order.
  void emit(std::ostringstream &os, int ind, int lookahead) const {
    std::string pad(ind, ' ');
    std::vector<size_t> order(stmts_.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return stmts_[a].key < stmts_[b].key; });
    std::vector<size_t> loads;
    for (size_t i = 0; i < stmts_.size(); ++i)
      if (stmts_[i].cat == Cat::Index) os << pad << stmts_[i].text << "\n";
    for (size_t i : order)
      if (stmts_[i].cat == Cat::Load) loads.push_back(i);
    for (size_t i = 0; i < stmts_.size(); ++i)
      if (stmts_[i].cat == Cat::Prefetch) os << pad << stmts_[i].text << "\n";
    // Ring loads: issued (cp.async into slot r % ring_) where a register load
    // would be issued, read back where it would be consumed after waiting for
    // its copy group.  At most `lookahead` loads are in flight, so with
    // lookahead <= ring_ a slot is read before it is reused.
    if (ring_ > 0 && lookahead > ring_) lookahead = ring_;
    size_t emitted = 0, seen = 0;
    int ring_issued = 0;
    auto slot = [&](int r) { return "cc_ring[" + std::to_string(r % ring_) + " * blockDim.x + threadIdx.x]"; };
    auto emit_loads_to = [&](size_t n) {
      if (n > loads.size()) n = loads.size();
      // batched loads: top up in whole groups so neighbours share a block
      if (batch_loads_ && n > emitted) n = std::min(loads.size(), emitted + (n - emitted + kLoadBatch - 1) / kLoadBatch * kLoadBatch);
      while (emitted < n) {
        const Stmt &l = stmts_[loads[emitted++]];
        if (l.batchable) {
          // up to kLoadBatch consecutive loads under the same condition: one
          // predicate for all of them
          std::vector<const Stmt *> run{&l};
          while (emitted < n && run.size() < (size_t)kLoadBatch) {
            const Stmt &m = stmts_[loads[emitted]];
            if (!m.batchable || m.ok != l.ok) break;
            run.push_back(&m);
            ++emitted;
          }
          const int k = (int)run.size();
          for (const Stmt *m : run) os << pad << "float " << m->var << " = " << lit_code(m->ubits) << ";\n";
          os << pad << "asm volatile(\"{\\n .reg .pred q;\\n setp.ne.b32 q, %" << 2 * k << ", 0;\\n";
          for (int j = 0; j < k; ++j) os << " @q ld.global.nc.f32 %" << j << ", [%" << k + j << "];\\n";
          os << "}\\n\"\n" << pad << "    : ";
          for (int j = 0; j < k; ++j) os << (j ? ", " : "") << "\"+f\"(" << run[j]->var << ")";
          os << "\n" << pad << "    : ";
          for (int j = 0; j < k; ++j) os << "\"l\"(" << run[j]->ptr << "), ";
          os << "\"r\"((int)(" << (l.ok.empty() ? std::string("1") : l.ok) << ")));\n";
          continue;
        }
        if (l.ring < 0) {
          os << pad << l.text << "\n";
          continue;
        }
        const std::string src = l.ok.empty() ? l.ptr : "(" + l.ok + ") ? " + l.ptr + " : " + l.base;
        os << pad << "cc_cp4(&" << slot(l.ring) << ", " << src << ", " << (l.ok.empty() ? "1" : "(" + l.ok + ")")
           << ");\n";
        ++ring_issued;
      }
    };
    for (size_t i : order) {
      const Stmt &s = stmts_[i];
      if (s.cat == Cat::Index || s.cat == Cat::Prefetch) continue;
      if (s.cat == Cat::Load) {
        ++seen;
        // a ring load waits here, so first fill the window (one short of the
        // ring: this load's slot is still unread)
        emit_loads_to(s.ring >= 0 && lookahead > 1 ? seen - 1 + (size_t)lookahead : seen);
        if (s.ring >= 0)
          os << pad << "cc_cp_wait<" << (ring_issued - s.ring - 1) << ">();\n"
             << pad << "const float " << s.var << " = " << slot(s.ring) << ";\n";
        continue;
      }
      emit_loads_to(seen + (size_t)(lookahead > 0 ? lookahead : 0));
      os << pad << s.text << "\n";
    }
    emit_loads_to(loads.size());
  }

  // Parameters read only at indices that depend on no output coordinate, of at
  // most `max_bytes` together, are copied into shared memory once per block
  // (`cc_sp<k>`) and read from there: a broadcast shared load instead of a
  // global load through L1 for every use.  Returns (parameter, floats) pairs.
  std::vector<std::pair<int, int64_t>> stage_uniform_params(int64_t max_bytes) {
    std::vector<std::pair<int, int64_t>> staged;
    std::set<int> chosen;
    int64_t total = 0;
    // Worth it only when such loads dominate: the copy and its barrier delay
    // the first per-thread load, which a short one-wave kernel feels.
    int uniform_loads = 0, varying_loads = 0;
    for (const Stmt &st : stmts_) {
      if (st.uparam >= 0 && !varying_params_.count(st.uparam)) ++uniform_loads;
      if (st.cat == Cat::Load) ++varying_loads;
    }
    if (uniform_loads < 2 * varying_loads) return staged;
    for (const Stmt &st : stmts_) {
      if (st.uparam < 0 || varying_params_.count(st.uparam) || chosen.count(st.uparam)) continue;
      const IrNode &p = ir_.nodes[ir_.param_nodes[st.uparam]];
      int64_t elems = 1;
      for (int64_t d : p.dims) elems *= d;
      if (elems <= 0 || total + 4 * elems > max_bytes) continue;
      total += 4 * elems;
      chosen.insert(st.uparam);
      staged.emplace_back(st.uparam, elems);
    }
    read_staged(staged);
    return staged;
  }
  // Reads these staged parameters from their shared-memory copies.
  void read_staged(const std::vector<std::pair<int, int64_t>> &staged) {
    std::set<int> chosen;
    for (auto &sp : staged) chosen.insert(sp.first);
    for (Stmt &st : stmts_) {
      if (st.uparam < 0 || !chosen.count(st.uparam)) continue;
      const std::string sp = "cc_sp" + std::to_string(st.uparam) + "[" + st.uoff + "]";
      st.text = "const float " + st.var + " = " +
                (st.ok.empty() ? sp : "(" + st.ok + ") ? " + sp + " : " + lit_code(st.ubits)) + ";";
    }
  }

  // Stage zero-padded loads that vary per thread through a shared-memory ring
  // of `slots` entries per thread (0: registers only).
  void set_ring(int slots) { ring_ = slots; }
  // Merge statements with identical right-hand sides (the frames of several
  // points per thread share index arithmetic, loads and arithmetic).
  void set_merge(bool on) { merge_ = on; }
  // Emit scalar predicated loads of one condition in groups of kLoadBatch,
  // one predicate per group.
  void set_batch_loads(bool on) { batch_loads_ = on; }
  void set_lanes(bool on) { lanes_ = on; }
  // Group reads of the same 16 bytes into float4 loads (needs merging on).
  void set_vector_loads(bool on) { vec_loads_ = on; }
  // Parameters with shared-memory copies (cc_sp<k>, 16-byte aligned).
  void set_staged(const std::vector<std::pair<int, int64_t>> &staged) {
    for (auto &sp : staged) staged_.insert(sp.first);
  }
  int vector_loads() const { return vector_loads_; }
  // Statements generated next belong to point k of `points`: statement i of
  // every point is ordered as (i, k), so the points advance together.
  void set_point(int k, int points) {
    point_ = k;
    points_ = points;
    pos_ = 0;
  }
  int ring_loads() const { return ring_loads_; }

  bool uses_fp64() const { return fp64_; }

 private:
  std::string fresh() { return "_" + std::to_string(next_var_++); }
  // With merging on, a statement whose right-hand side (`key`) was emitted
  // before reuses that variable: `v` becomes its name and true is returned.
  // The merged statement moves up to where this point would have created it,
  // so the points' statements interleave (short live ranges) and every
  // statement still follows its operands.
  bool reuse(const std::string &key, std::string &v) {
    if (!merge_) return false;
    auto it = merged_.find(key);
    if (it == merged_.end()) {
      merged_.emplace(key, v);
      pending_var_ = v;
      return false;
    }
    v = it->second;
    const int64_t here = pos_++ * points_ + point_;
    auto s = stmt_of_.find(v);
    if (s != stmt_of_.end() && stmts_[s->second].key > here) stmts_[s->second].key = here;
    return true;
  }
  void add(Cat c, std::string t) {
    Stmt st{c, std::move(t)};
    push(std::move(st));
  }
  void push(Stmt st) {
    st.key = pos_++ * points_ + point_;
    if (!pending_var_.empty() && st.cat != Cat::Prefetch) {
      stmt_of_[pending_var_] = stmts_.size();  // the statement defining the last unmerged value
      pending_var_.clear();
    }
    stmts_.push_back(std::move(st));
  }

  // A read whose innermost index is a constant c, from a parameter whose
  // innermost extent is a multiple of 4, becomes component c % 4 of a float4
  // load at c - c % 4 that the other reads of the same group share: one
  // 16-byte load where a view splits a short innermost axis (channels, say)
  // into separate reads.  Needs 16-byte aligned inputs (cc_ew_vl).
  // A thread-independent read of a staged parameter groups the same way into
  // a float4 read of its (16-byte aligned) shared-memory copy.
  // A thread-independent read of an unstaged parameter stays a global load,
  // emitted where it is used like the scalar one (`windowed` false).
  bool vector_load(const IrNode &p, const std::vector<std::string> &idx, const std::vector<std::string> &row_ok,
                   const std::vector<std::pair<bool, int64_t>> &row_const, bool global, bool windowed,
                   std::string &v) {
    const int r = (int)p.dims.size();
    if (r == 0 || p.dims[r - 1] % 4 != 0 || !row_const[r - 1].first) return false;
    const int64_t ci = row_const[r - 1].second;
    if (ci < 0 || ci >= p.dims[r - 1]) return false;
    int64_t total = 1;
    for (int64_t d : p.dims) total *= d;
    const bool wide = total >= (int64_t(1) << 31);
    std::string ok;
    for (int y = 0; y < r - 1; ++y)
      if (!row_ok[y].empty()) ok += std::string(ok.empty() ? "" : " && ") + row_ok[y];
    const std::string D = std::to_string(p.dims[r - 1]) + (wide ? "LL" : "");
    std::string prefix = r == 1 ? std::string() : offset_expr(std::vector<int64_t>(p.dims.begin(), p.dims.end() - 1),
                                                                std::vector<std::string>(idx.begin(), idx.end() - 1));
    std::string off = r == 1 ? std::to_string(ci - ci % 4)
                             : "(" + std::string(wide ? "(cc_i64)" : "") + prefix + ") * " + D + " + " +
                                   std::to_string(ci - ci % 4);
    const std::string ptr = global ? "in" + std::to_string(p.param_index) + " + " + off
                                   : "reinterpret_cast<const float4 *>(cc_sp" + std::to_string(p.param_index) + ")[(" +
                                         off + ") / 4]";
    std::string q = "_q" + std::to_string(next_var_++);
    if (!reuse("G " + ptr + " " + ok + " " + lit_code(p.bits), q)) {
      const std::string pad = lit_code(p.bits);
      const std::string pad4 = "make_float4(" + pad + ", " + pad + ", " + pad + ", " + pad + ")";
      if (global)
        add(windowed ? Cat::Load : Cat::Compute, "float4 " + q + " = " + pad4 + "; cc_ld4(" + q + ", " + ptr + ", " +
                                                     (ok.empty() ? std::string("1") : "(" + ok + ")") + ");");
      else
        add(Cat::Compute, "const float4 " + q + " = " + (ok.empty() ? ptr : "(" + ok + ") ? " + ptr + " : " + pad4) +
                              ";");
      ++vector_loads_;
    }
    // merged through the group, so a merged component moves up only after it
    const std::string comp = q + "." + "xyzw"[ci % 4];
    if (!reuse("C " + comp, v)) add(Cat::Compute, "const float " + v + " = " + comp + ";");
    return true;
  }

  // One index variable per source dimension, the way ArrayView.extract
  // computes it (OpenCLKernelBuilder.scala:348-411); returns the bounds
  // condition ("" when every row is constant-zero and no check applies).
  // row_const: per row, whether the index is a known integer and its value
  // (integral coefficients on known index variables only).
  std::string index_rows(const IrNode &node, const std::vector<int64_t> &dims, const Frame &f,
                         std::vector<std::string> &idx, std::vector<std::string> *row_ok = nullptr,
                         std::vector<std::pair<bool, int64_t>> *row_const = nullptr) {
    const int rows = (int)dims.size();
    const int cols = node.cols;
    std::string ok;
    for (int y = 0; y < rows; ++y) {
      std::string sum;
      bool any = false;
      double c = node.m[(size_t)y * cols + cols - 1];
      for (int x = 0; x < cols - 1 && !f.goff.empty(); ++x) c += node.m[(size_t)y * cols + x] * (double)f.goff[x];
      for (int x = 0; x < cols; ++x) {
        double s = x < cols - 1 ? node.m[(size_t)y * cols + x] : c;
        if (s == 0.0) continue;
        std::string term;
        if (x < cols - 1) {
          term = (s == 1.0) ? f.gid[x] : f.gid[x] + " * " + literal(s);
        } else {
          term = literal(s);
        }
        sum += (any ? " + " : "") + term;
        any = true;
      }
      std::string name = "_i" + std::to_string(next_var_++);
      const std::string rhs = any ? "(int)(" + sum + ")" : "0";
      if (!reuse("I " + rhs, name)) {
        bool row_uniform = true;
        for (int x = 0; x < cols - 1; ++x)
          if (node.m[(size_t)y * cols + x] != 0.0 && !uniform_.count(f.gid[x])) row_uniform = false;
        if (row_uniform) uniform_.insert(name);
        add(Cat::Index, "const int " + name + " = " + rhs + ";");
      }
      // the index as a compile-time integer, when the row has one
      bool known = c == (double)(int64_t)c;
      double kv = c;
      for (int x = 0; x < cols - 1 && known; ++x) {
        const double s = node.m[(size_t)y * cols + x];
        if (s == 0.0) continue;
        if (s != (double)(int64_t)s || x >= (int)f.gknown.size() || !f.gknown[x]) {
          known = false;
        } else {
          kv += s * (double)f.gval[x];
        }
      }
      std::string cond;
      if (!any) {
        if (dims[y] == 0) cond = "false";
      } else if (known && f.gknown.size() > 0) {
        // a known index through a view: its bounds test is decided here
        if (kv < 0.0 || kv >= (double)dims[y]) cond = "false";
      } else {
        cond = "(" + name + " >= 0) && (" + name + " < " + std::to_string(dims[y]) + ")";
      }
      if (!cond.empty()) ok += std::string(ok.empty() ? "" : " && ") + cond;
      if (row_ok) row_ok->push_back(cond);
      if (row_const) row_const->emplace_back(known, known ? (int64_t)kv : 0);
      idx.push_back(name);
    }
    return ok;
  }

  std::string literal(double s) {
    std::string t = decimal_format3(s);
    if (t.find('.') != std::string::npos) fp64_ = true;
    if (t[0] == '-') return "(" + t + ")";
    return t;
  }

  static std::string offset_expr(const std::vector<int64_t> &dims, const std::vector<std::string> &idx) {
    if (dims.empty()) return "0";
    int64_t total = 1;
    for (int64_t d : dims) total *= d;
    bool wide = total >= (int64_t(1) << 31);
    std::string e = wide ? "(cc_i64)" + idx[0] : idx[0];
    for (size_t i = 1; i < dims.size(); ++i) {
      e = "(" + e + " * " + std::to_string(dims[i]) + (wide ? "LL" : "") + " + " + idx[i] + ")";
    }
    return e;
  }

  const Ir &ir_;
  bool contig_;
  bool asm_loads_;
  int64_t prefetch_min_bytes_;
  bool shared_transcendentals_;
  // Lane-generic contiguous code: every value has the template type T and
  // every operation other than + - * / and negation goes through an
  // overloaded cc_ helper (cc_exp, cc_fma, cc_min, ...), so one body serves a
  // scalar and a several-lane evaluation with the same per-lane arithmetic.
  bool lanes_ = false;
  std::string ty() const { return lanes_ ? "T" : "float"; }
  bool fp64_ = false;
  int next_var_ = 0;
  int next_frame_ = 1;
  bool merge_ = false;
  bool batch_loads_ = false;
  static constexpr int kLoadBatch = 8;
  bool vec_loads_ = false;
  std::set<int> staged_;
  int vector_loads_ = 0;
  std::map<std::string, std::string> merged_;     // right-hand side -> variable
  std::map<std::string, size_t> stmt_of_;         // variable -> defining statement
  std::string pending_var_;
  int64_t pos_ = 0;  // statement events of the current point
  int point_ = 0, points_ = 1;
  std::map<std::pair<int, int>, std::string> memo_;
  std::vector<Stmt> stmts_;
  std::set<std::string> uniform_;  // index variables that depend on no output coordinate
  int ring_ = 0;
  int ring_loads_ = 0;
  std::set<int> varying_params_;  // parameters read at least once at a per-thread index
  bool fma_ = false;              // contract a product operand of + / - into fmaf
};

bool is_contiguous_identity(const IrNode &x, const IrNode &p, const std::vector<int64_t> &out_shape) {
  if (p.dims != out_shape) return false;
  const int rows = (int)p.dims.size();
  const int cols = x.cols;
  if (cols != rows + 1) return false;
  for (int y = 0; y < rows; ++y)
    for (int c = 0; c < cols; ++c)
      if (x.m[(size_t)y * cols + c] != (c == y ? 1.0 : 0.0)) return false;
  return true;
}

}  // namespace

namespace {

bool matrix_is(const IrNode &n, std::initializer_list<double> want) {
  if (n.m.size() != want.size()) return false;
  size_t i = 0;
  for (double w : want)
    if (n.m[i++] != w) return false;
  return true;
}

}  // namespace

bool match_contraction(const Ir &ir, Contraction *out) {
  if (ir.kind != ProgramKind::Elementwise || ir.out_shape.size() != 2) return false;
  // the left spine of additions: ((t0 + t1) + t2) + ...
  std::vector<int> terms;
  int node = ir.root;
  while (ir.nodes[node].kind == NodeKind::Binary && ir.nodes[node].op == (uint8_t)BinOp::Add) {
    terms.push_back(ir.nodes[node].b);
    node = ir.nodes[node].a;
  }
  terms.push_back(node);
  if (terms.size() < 2) return false;
  std::reverse(terms.begin(), terms.end());
  const int64_t I = ir.out_shape[0], K = ir.out_shape[1], J = (int64_t)terms.size();
  int sub = -1;
  for (int64_t j = 0; j < J; ++j) {
    const IrNode &v = ir.nodes[terms[j]];
    if (v.kind != NodeKind::View || v.cols != 3) return false;
    if (v.dims != std::vector<int64_t>{I, J, K}) return false;
    if (!matrix_is(v, {1, 0, 0, 0, 0, (double)j, 0, 1, 0})) return false;
    if (sub < 0) sub = v.a;
    if (v.a != sub) return false;
  }
  const IrNode &mul = ir.nodes[sub];
  if (mul.kind != NodeKind::Binary || mul.op != (uint8_t)BinOp::Mul) return false;
  int a_in = -1, b_in = -1;
  for (int operand : {mul.a, mul.b}) {
    const IrNode &x = ir.nodes[operand];
    if (x.kind != NodeKind::Extract || x.cols != 4) return false;
    const IrNode &p = ir.nodes[x.a];
    if (p.dims == std::vector<int64_t>{I, J} && matrix_is(x, {1, 0, 0, 0, 0, 1, 0, 0})) {
      a_in = p.param_index;
    } else if (p.dims == std::vector<int64_t>{1, J, K} &&
               matrix_is(x, {0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0})) {
      b_in = p.param_index;
    } else if (p.dims == std::vector<int64_t>{J, K} && matrix_is(x, {0, 1, 0, 0, 0, 0, 1, 0})) {
      b_in = p.param_index;
    } else {
      return false;
    }
  }
  if (a_in < 0 || b_in < 0) return false;
  if (I > INT32_MAX || J > INT32_MAX || K > INT32_MAX) return false;
  out->a_input = a_in;
  out->b_input = b_in;
  out->m = I;
  out->k = J;
  out->n = K;
  return true;
}

namespace {

// Row y of view matrix `m` (cols columns) selects coordinate y and nothing else.
bool row_selects(const std::vector<double> &m, int cols, int y, int coord) {
  for (int c = 0; c < cols; ++c)
    if (m[(size_t)y * cols + c] != (c == coord ? 1.0 : 0.0)) return false;
  return true;
}

// The last row of a split's view matrix: no coordinate, the constant j.
bool row_is_constant(const std::vector<double> &m, int cols, int y, double value) {
  for (int c = 0; c + 1 < cols; ++c)
    if (m[(size_t)y * cols + c] != 0.0) return false;
  return m[(size_t)y * cols + cols - 1] == value;
}

// A read of a tensor of shape [1, ..., 1, J] at the frame's last coordinate:
// the rows of the size-one dimensions have no term (index 0, as a broadcast
// reads them) and the last row selects coordinate frame_rank - 1.
bool is_column_read(const IrNode &x, const IrNode &p, int64_t J, int frame_rank) {
  if (p.dims.empty() || p.dims.back() != J) return false;
  const int rows = (int)p.dims.size(), cols = frame_rank + 1;
  if (x.cols != cols || (int)x.m.size() != rows * cols) return false;
  for (int y = 0; y + 1 < rows; ++y) {
    if (p.dims[y] != 1) return false;
    for (int c = 0; c < cols; ++c)
      if (x.m[(size_t)y * cols + c] != 0.0) return false;
  }
  return row_selects(x.m, cols, rows - 1, frame_rank - 1);
}

}  // namespace

bool match_row_fold(const Ir &ir, RowFold *out, std::string *why) {
  auto no = [&](const char *m) {
    if (why) *why = m;
    return false;
  };
  if (ir.kind != ProgramKind::Elementwise) return no("not an elementwise program");
  std::vector<int> terms;
  int node = ir.root;
  while (ir.nodes[node].kind == NodeKind::Binary && ir.nodes[node].op == (uint8_t)BinOp::Add) {
    terms.push_back(ir.nodes[node].b);
    node = ir.nodes[node].a;
  }
  terms.push_back(node);
  const int64_t J = (int64_t)terms.size();
  if (J < kRowFoldMinTerms) return no("fewer terms than the fold skeleton takes");
  std::reverse(terms.begin(), terms.end());
  const int out_rank = (int)ir.out_shape.size();
  std::vector<int64_t> frame = ir.out_shape;
  frame.push_back(J);
  const int cols = out_rank + 1;
  // every term: the same fused tensor (a View of one node) or the same parameter,
  // of shape `frame`, at coordinates (g, j)
  const IrNode &first = ir.nodes[terms[0]];
  if (first.kind != NodeKind::View && first.kind != NodeKind::Extract) return no("terms are not views");
  const bool fused = first.kind == NodeKind::View;
  for (int64_t j = 0; j < J; ++j) {
    const IrNode &v = ir.nodes[terms[j]];
    if (v.kind != first.kind || v.a != first.a || v.cols != cols) return no("terms differ");
    const std::vector<int64_t> &dims = fused ? v.dims : ir.nodes[v.a].dims;
    if (dims != frame) return no("terms do not split the last dimension");
    for (int y = 0; y < out_rank; ++y)
      if (!row_selects(v.m, cols, y, y)) return no("terms are not read at the output's coordinates");
    if (!row_is_constant(v.m, cols, out_rank, (double)j)) return no("terms are not in split order");
  }
  RowFold rf;
  rf.rows = 1;
  for (int64_t d : ir.out_shape) rf.rows *= d;
  rf.cols = J;
  rf.is_row.assign(ir.n_params, false);
  std::vector<bool> is_col(ir.n_params, false);
  if (!fused) {
    rf.term = terms[0];
    rf.term_frame = ir.out_shape;
    rf.is_row[ir.nodes[first.a].param_index] = true;
  } else {
    rf.term = first.a;
    rf.term_frame = frame;
    // the template: literals, operators and reads of row or column inputs
    std::vector<int> stack{first.a};
    std::set<int> seen;
    while (!stack.empty()) {
      const int n = stack.back();
      stack.pop_back();
      if (!seen.insert(n).second) continue;
      const IrNode &x = ir.nodes[n];
      switch (x.kind) {
        case NodeKind::Literal: break;
        case NodeKind::Unary: stack.push_back(x.a); break;
        case NodeKind::Binary:
          stack.push_back(x.a);
          stack.push_back(x.b);
          break;
        case NodeKind::Extract: {
          const IrNode &p = ir.nodes[x.a];
          const int fc = (int)frame.size() + 1;
          if (x.cols != fc) return no("template read of another rank");
          if (is_contiguous_identity(x, p, frame)) {
            rf.is_row[p.param_index] = true;
          } else if (is_column_read(x, p, J, (int)frame.size())) {
            is_col[p.param_index] = true;
          } else {
            return no("template reads an input through a view");
          }
          break;
        }
        default: return no("template holds a nested view or tuple");
      }
    }
  }
  for (int k = 0; k < ir.n_params; ++k) {
    if (rf.is_row[k] && is_col[k]) return no("an input read both as a row and as a column");
    if (rf.is_row[k]) rf.row_inputs.push_back(k);
  }
  if (rf.row_inputs.empty()) return no("no row input");
  if ((int)rf.row_inputs.size() > kRowFoldMaxInputs) return no("more row inputs than the ring stages");
  if (J % 4 != 0) return no("rows are not a multiple of 16 bytes");
  if (rf.rows >= (int64_t(1) << 31) || J >= (int64_t(1) << 31)) return no("too many rows or terms for TMA coordinates");
  if (out) *out = rf;
  return true;
}

int row_fold_stages(int row_inputs, int requested) {
  const int per_stage = row_inputs * kRowFoldRows * 128;
  if (requested >= 2 && requested <= 16 && requested * per_stage + 1024 <= 200 * 1024) return requested;
  int s = (96 * 1024) / (per_stage > 0 ? per_stage : 1);
  return s < 2 ? 2 : s > 12 ? 12 : s;
}

int row_fold_smem_bytes(int row_inputs, int stages) { return stages * row_inputs * kRowFoldRows * 128 + 1024; }

std::string row_fold_source(const Ir &ir, const RowFold &rf) {
  Generator gen(ir, true, false, -1, false);
  std::ostringstream body;
  Frame f0{0, {}, rf.term_frame};
  const std::string r = gen.gen(rf.term, f0);
  gen.emit(body, 2, 0);
  const int n = ir.n_params, nin = (int)rf.row_inputs.size(), S = row_fold_stages(nin, rf.stages);
  std::vector<int> slot(n, -1);  // parameter -> row-input slot
  for (int i = 0; i < nin; ++i) slot[rf.row_inputs[i]] = i;
  std::ostringstream o;
  o << "// generated by compute.scala_gb300 for sm_103a: inner-axis fold of " << rf.cols << " terms per output\n"
    << kPrelude << "\n";
  o << "#define CC_RF_ROWS " << kRowFoldRows << "\n#define CC_RF_NIN " << nin << "\n#define CC_RF_STAGES " << S
    << "\n#define CC_RF_TILE (CC_RF_ROWS * 128)\n\n";
  // one term of the fold, from its inputs' values at (g, j)
  o << "__device__ __forceinline__ float cc_rf_term(";
  for (int k = 0; k < n; ++k) o << (k ? ", " : "") << "const float a" << k;
  o << ") {\n" << body.str() << "  return " << r << ";\n}\n\n";
  std::ostringstream params;
  for (int i = 0; i < nin; ++i) params << "const __grid_constant__ cc_tensor_map tm" << i << ", ";
  for (int k = 0; k < n; ++k) params << "const float *__restrict__ in" << k << ", ";
  params << "float *__restrict__ out, long long rows, int cols, int *__restrict__ err";
  // the term at column expression `j` with row-input values `val(i)`
  auto call = [&](const std::function<std::string(int)> &val, const std::string &j) {
    std::string s = "cc_rf_term(";
    for (int k = 0; k < n; ++k) {
      if (k) s += ", ";
      s += slot[k] >= 0 ? val(slot[k]) : "__ldg(in" + std::to_string(k) + " + " + j + ")";
    }
    return s + ")";
  };
  static const char *comp[] = {"x", "y", "z", "w"};
  // ---- cc_rowfold: TMA tiles of 64 rows x 32 floats (128 bytes, swizzled), one per row input
  o << "// Each block folds CC_RF_ROWS outputs, one per thread, in the order j = 0, 1, 2, ...\n"
       "// Thread 0 keeps CC_RF_STAGES tiles of every row input in flight (TMA, 128-byte swizzle:\n"
       "// 16-byte chunk c of tile row r sits at chunk c ^ (r % 8), so eight threads reading their\n"
       "// own rows' chunk c hit eight different bank groups).\n";
  o << "extern \"C\" __global__ void __launch_bounds__(CC_RF_ROWS) cc_rowfold(" << params.str() << ") {\n"
    << "  extern __shared__ unsigned char cc_rf_raw[];\n"
    << "  __shared__ __align__(8) unsigned long long cc_rf_full[CC_RF_STAGES];\n"
    << "  __shared__ int cc_rf_abort;\n"
    << "  unsigned char *const ring = (unsigned char *)(((unsigned long long)cc_rf_raw + 1023ull) & ~1023ull);\n"
    << "  const int tid = threadIdx.x;\n"
    << "  const long long row0 = (long long)blockIdx.x * CC_RF_ROWS;\n"
    << "  const int ntiles = (cols + 31) >> 5;\n"
    << "  if (tid == 0) {\n"
    << "    for (int s = 0; s < CC_RF_STAGES; ++s) cc_mbar_init(cc_smem_addr(&cc_rf_full[s]), 1);\n"
    << "    cc_mbar_init_fence();\n"
    << "    cc_rf_abort = 0;\n"
    << "  }\n"
    << "  __syncthreads();\n"
    << "  cc_pdl_wait_then_release();\n";
  std::ostringstream issue;
  issue << "      const unsigned bar = cc_smem_addr(&cc_rf_full[(u) % CC_RF_STAGES]);\n"
        << "      cc_mbar_expect_tx(bar, CC_RF_NIN * CC_RF_TILE);\n";
  for (int i = 0; i < nin; ++i)
    issue << "      cc_tma_load_2d(cc_smem_addr(ring + ((u) % CC_RF_STAGES * CC_RF_NIN + " << i
          << ") * CC_RF_TILE), &tm" << i << ", (u) << 5, (int)row0, bar);\n";
  o << "  if (tid == 0)\n    for (int u = 0; u < CC_RF_STAGES && u < ntiles; ++u) {\n" << issue.str() << "    }\n";
  o << "  float acc = 0.0f;\n"
    << "  int t = 0;\n"
    << "  for (; t < ntiles; ++t) {\n"
    << "    const int s = t % CC_RF_STAGES;\n"
    << "    if (!cc_mbar_wait_bounded(cc_smem_addr(&cc_rf_full[s]), (unsigned)((t / CC_RF_STAGES) & 1), 2000000000ull)) {\n"
    << "      atomicCAS(err, 0, " << kRowFoldWaitCode << ");\n"
    << "      cc_rf_abort = 1;\n"
    << "    }\n"
    << "    const unsigned char *tile = ring + s * CC_RF_NIN * CC_RF_TILE + tid * 128;\n"
    << "    const int j0 = t << 5;\n"
    << "    if (t > 0 && cols - j0 >= 32) {\n";
  for (int g = 0; g < 2; ++g) {
    // g = 0: a full tile, no bounds; g = 1: the first or a partial tile
    if (g == 1) o << "    } else {\n      const int hi = cols - j0 < 32 ? cols - j0 : 32;\n";
    o << "#pragma unroll\n      for (int c = 0; c < 8; ++c) {\n"
      << "        const int off = (c ^ (tid & 7)) << 4;\n";
    for (int i = 0; i < nin; ++i)
      o << "        const float4 q" << i << " = *reinterpret_cast<const float4 *>(tile + " << i
        << " * CC_RF_TILE + off);\n";
    for (int e = 0; e < 4; ++e) {
      const std::string j = "(j0 + c * 4 + " + std::to_string(e) + ")";
      const std::string term = call([&](int i) { return "q" + std::to_string(i) + "." + comp[e]; }, j);
      if (g == 0) {
        o << "        acc = acc + " << term << ";\n";
      } else {
        o << "        if (c * 4 + " << e << " < hi) {\n"
          << "          const float v = " << term << ";\n"
          << "          acc = " << j << " == 0 ? v : acc + v;\n"
          << "        }\n";
      }
    }
    o << "      }\n";
  }
  o << "    }\n"
    << "    __syncthreads();\n"
    << "    if (cc_rf_abort) break;\n"
    << "    if (tid == 0 && t + CC_RF_STAGES < ntiles) {\n"
    << "      const int u = t + CC_RF_STAGES;\n"
    << issue.str()
    << "    }\n"
    << "  }\n"
    << "  if (cc_rf_abort) {\n"
    << "    // loads still in flight land before the block's shared memory is given up\n"
    << "    if (tid == 0)\n"
    << "      for (int u = t; u < ntiles && u < t + CC_RF_STAGES; ++u)\n"
    << "        cc_mbar_wait_bounded(cc_smem_addr(&cc_rf_full[u % CC_RF_STAGES]), (unsigned)((u / CC_RF_STAGES) & 1), "
       "100000000ull);\n"
    << "    return;\n"
    << "  }\n"
    << "  if (row0 + tid < rows) out[row0 + tid] = acc;\n"
    << "}\n\n";
  // ---- cc_rowfold_plain: the same fold with direct loads (row inputs not 16-byte aligned)
  o << "extern \"C\" __global__ void __launch_bounds__(CC_RF_ROWS) cc_rowfold_plain(" << params.str() << ") {\n"
    << "  cc_pdl_wait_then_release();\n"
    << "  const long long row = (long long)blockIdx.x * CC_RF_ROWS + threadIdx.x;\n"
    << "  if (row >= rows) return;\n";
  for (int i = 0; i < nin; ++i)
    o << "  const float *r" << i << " = in" << rf.row_inputs[i] << " + row * (long long)cols;\n";
  const std::string t0 = call([&](int i) { return "__ldg(r" + std::to_string(i) + ")"; }, "0");
  const std::string tj = call([&](int i) { return "__ldg(r" + std::to_string(i) + " + j)"; }, "j");
  o << "  float acc = " << t0 << ";\n"
    << "  for (int j = 1; j < cols; ++j) acc = acc + " << tj << ";\n"
    << "  out[row] = acc;\n"
    << "}\n";
  return o.str();
}

bool is_batchable(const Ir &ir, std::string *why) {
  auto no = [&](const char *m) {
    if (why) *why = m;
    return false;
  };
  if (ir.kind != ProgramKind::Elementwise) return no("only elementwise programs are batched");
  if (ir.nodes[ir.root].kind == NodeKind::Tuple) return no("tuple-valued programs are not batched");
  if (ir.n_params > kBatchMaxInputs) return no("a batched program has at most 4 inputs");
  for (const IrNode &n : ir.nodes) {
    if (n.kind == NodeKind::View) return no("a batched program reads its inputs without views");
    if (n.kind == NodeKind::Extract && !is_contiguous_identity(n, ir.nodes[n.a], ir.out_shape))
      return no("a batched program reads its inputs without views");
  }
  return true;
}

std::string point_function(const Ir &ir, const std::string &name, bool inline_it, bool shared_transcendentals,
                           bool lanes) {
  Generator gen(ir, true, false, -1, shared_transcendentals);
  gen.set_lanes(lanes);
  std::ostringstream body;
  Frame f0{0, {}, ir.out_shape};
  std::string r = gen.gen(ir.root, f0);
  gen.emit(body, 2, 0);
  std::ostringstream o;
  const char *ty = lanes ? "T" : "float";
  if (lanes) o << "template <class T> ";
  o << "__device__ " << (inline_it ? "__forceinline__" : "__noinline__") << " " << ty << " " << name << "(";
  for (int i = 0; i < kBatchMaxInputs; ++i) o << (i ? ", " : "") << ty << " a" << i;
  o << ") {\n" << body.str() << "  return " << r << ";\n}\n";
  return o.str();
}

int choose_min_blocks(int64_t domain, int block, int sm_count, int override_blocks) {
  if (override_blocks > 0) return override_blocks;
  if (sm_count <= 0) return 0;
  const int64_t blocks = (domain + block - 1) / block;
  const int64_t per_sm = (blocks + sm_count - 1) / sm_count;
  int64_t max_per_sm = 2048 / block;
  if (max_per_sm > 32) max_per_sm = 32;  // resident blocks per SM
  if (per_sm <= max_per_sm) return (int)(per_sm < 1 ? 1 : per_sm);
  return 4;
}

namespace {

bool program_is_contiguous(const Ir &ir) {
  const IrNode &root = ir.nodes[ir.root];
  if (root.kind == NodeKind::Tuple) return false;
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  if (domain <= 0) return false;
  for (const IrNode &n : ir.nodes) {
    if (n.kind == NodeKind::View) return false;
    if (n.kind == NodeKind::Extract && !is_contiguous_identity(n, ir.nodes[n.a], ir.out_shape)) return false;
  }
  return true;
}

}  // namespace

std::string contiguous_structure_key(const Ir &ir) {
  if (!program_is_contiguous(ir)) return std::string();
  std::ostringstream o;
  o << "contiguous " << (ir.kind == ProgramKind::Sum ? "sum" : "ew") << "\n";
  char b[16];
  for (const IrNode &n : ir.nodes) {
    switch (n.kind) {
      case NodeKind::Param:
        snprintf(b, sizeof b, "%08x", n.bits);
        o << "p " << b << "\n";
        break;
      case NodeKind::Literal:
        snprintf(b, sizeof b, "%08x", n.bits);
        o << "l " << b << "\n";
        break;
      case NodeKind::Extract: o << "x " << n.a << "\n"; break;
      case NodeKind::Unary: o << "u " << kUnNames[n.op] << " " << n.a << "\n"; break;
      case NodeKind::Binary: o << "b " << kBinNames[n.op] << " " << n.a << " " << n.b << "\n"; break;
      default: return std::string();
    }
  }
  o << "r " << ir.root << "\n";
  return o.str();
}

namespace {

// Output coordinates g0..g<rank-1> of linear index `lin` (row-major).  Below
// 2^31 points the arithmetic is 32-bit unsigned, whose division by a constant
// compiles to a multiply and shifts; larger domains divide in 64 bits.
std::string decode_coordinates(const std::vector<int64_t> &shape, int64_t domain, const std::string &pad) {
  std::ostringstream os;
  const int rank = (int)shape.size();
  const bool narrow = domain < (int64_t(1) << 31);
  os << pad << (narrow ? "unsigned int rem_ = (unsigned int)lin;\n" : "cc_i64 rem_ = lin;\n");
  for (int d = rank - 1; d >= 1; --d) {
    if (narrow) {
      os << pad << "const int g" << d << " = (int)(rem_ % " << shape[d] << "u);\n";
      os << pad << "rem_ /= " << shape[d] << "u;\n";
    } else {
      os << pad << "const int g" << d << " = (int)(rem_ % " << shape[d] << "LL);\n";
      os << pad << "rem_ /= " << shape[d] << "LL;\n";
    }
  }
  os << pad << "const int g0 = (int)rem_;\n";
  return os.str();
}

}  // namespace

namespace {
std::vector<int64_t> param_bytes_of(const Ir &ir) {
  std::vector<int64_t> out(ir.n_params, 0);
  for (const IrNode &n : ir.nodes)
    if (n.kind == NodeKind::Param && n.param_index >= 0 && n.param_index < ir.n_params) {
      int64_t b = 4;
      for (int64_t d : n.dims) b *= d;
      out[n.param_index] = b;
    }
  return out;
}
}  // namespace

Generated describe_program(const Ir &ir) {
  Generated g;
  g.n_inputs = ir.n_params;
  g.param_bytes = param_bytes_of(ir);
  const IrNode &root = ir.nodes[ir.root];
  g.tuple_len = root.kind == NodeKind::Tuple ? (int)root.elems.size() : 1;
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  g.domain = domain;
  g.out_elems = ir.kind == ProgramKind::Sum ? 1 : domain * g.tuple_len;
  g.has_vec4 = program_is_contiguous(ir);
  return g;
}

// Shared memory a generic kernel may use for copies of small parameters read at
// thread-independent indices.
constexpr int64_t kMaxStagedBytes = 16 * 1024;

int points_for(const Ir &ir, int requested) {
  const int rank = (int)ir.out_shape.size();
  if (requested <= 1 || rank == 0 || ir.kind != ProgramKind::Elementwise || program_is_contiguous(ir)) return 1;
  return ir.out_shape[rank - 1] % requested == 0 ? requested : 1;
}

Generated generate_cuda(const Ir &ir, const CodegenOptions &opt) {
  Generated g;
  g.n_inputs = ir.n_params;
  g.param_bytes = param_bytes_of(ir);
  const IrNode &root = ir.nodes[ir.root];
  g.tuple_len = root.kind == NodeKind::Tuple ? (int)root.elems.size() : 1;
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  g.domain = domain;
  g.out_elems = ir.kind == ProgramKind::Sum ? 1 : domain * g.tuple_len;
  const int rank = (int)ir.out_shape.size();

  // Contiguous: every value reachable from the root is a literal, an operator,
  // or an identity read of a parameter with the output's shape.
  bool contiguous = g.tuple_len == 1 && domain > 0;
  for (const IrNode &n : ir.nodes) {
    if (n.kind == NodeKind::View) contiguous = false;
    if (n.kind == NodeKind::Extract && !is_contiguous_identity(n, ir.nodes[n.a], ir.out_shape)) contiguous = false;
  }
  g.has_vec4 = contiguous;

  std::ostringstream src;
  src << "// generated by compute.scala_gb300 for sm_103a\n" << kPrelude << "\n";

  std::string params;
  for (int i = 0; i < ir.n_params; ++i) params += "const float *__restrict__ in" + std::to_string(i) + ", ";

  // Frame 0: output coordinates decoded from the linear index.
  Frame f0{0, {}, ir.out_shape};
  for (int d = 0; d < rank; ++d) f0.gid.push_back("g" + std::to_string(d));
  auto decode = [&](std::ostringstream &os, int ind) {
    std::string pad(ind, ' ');
    if (rank == 0) return;
    os << decode_coordinates(ir.out_shape, domain, pad);
  };

  const std::string block = std::to_string(opt.block);
  // launch bounds of the generic kernels (see choose_min_blocks)
  const std::string lb = opt.min_blocks > 0 ? block + ", " + std::to_string(opt.min_blocks) : block;
  bool fp64 = false;

  if (contiguous) {
    // The point function of the contiguous form: parameter values in, result out.
    Generator gen(ir, true);
    std::ostringstream body;
    std::string r = gen.gen(ir.root, f0);
    gen.emit(body, 2, 0);
    fp64 |= gen.uses_fp64();
    src << "__device__ __forceinline__ float cc_point(";
    for (int i = 0; i < ir.n_params; ++i) src << (i ? ", " : "") << "float a" << i;
    if (ir.n_params == 0) src << "void";
    src << ") {\n" << body.str() << "  return " << r << ";\n}\n\n";
  }

  // Generic per-point body (frame 0 at coordinates decoded from `lin`).
  std::ostringstream generic;
  std::vector<std::string> results;
  int ring_slots = 0;
  std::vector<std::pair<int, int64_t>> staged;
  {
    Generator gen(ir, false, opt.asm_loads, opt.prefetch_min_bytes);
    gen.set_ring(contiguous ? 0 : opt.smem_ring);  // contiguous programs use the float4 kernels
    decode(generic, 4);
    if (root.kind == NodeKind::Tuple) {
      for (int e : root.elems) results.push_back(gen.gen(e, f0));
    } else {
      results.push_back(gen.gen(ir.root, f0));
    }
    if (!contiguous) staged = gen.stage_uniform_params(kMaxStagedBytes);
    gen.emit(generic, 4, opt.smem_ring > 0 ? std::min(opt.load_lookahead, opt.smem_ring) : opt.load_lookahead);
    fp64 |= gen.uses_fp64();
    if (gen.ring_loads() > 0) ring_slots = opt.smem_ring;
  }
  // Several consecutive points per thread along the last output dimension
  // (non-contiguous elementwise programs whose last extent P divides): one
  // frame per point, the last coordinate offset by k, all generated with
  // merging, so index rows, loads and arithmetic that do not depend on the
  // offset (a weight read, say) are emitted once for the P points.
  const int P = points_for(ir, opt.points_per_thread);
  g.points_per_thread = P;
  // Returns the number of float4 loads of the body (`vec`: grouped loads).
  auto merged_body = [&](bool vec, std::ostringstream &os, std::vector<std::vector<std::string>> &res) {
    Generator mg(ir, false, opt.asm_loads, opt.prefetch_min_bytes);
    mg.set_merge(true);
    mg.set_vector_loads(vec);
    mg.set_batch_loads(vec && opt.batch_loads);
    if (vec) mg.set_staged(staged);
    decode(os, 4);
    res.assign(P, {});
    for (int k = 0; k < P; ++k) {
      mg.set_point(k, P);
      Frame fk{-1 - k, f0.gid, ir.out_shape, std::vector<int64_t>(rank, 0)};
      if (rank > 0) fk.goff[rank - 1] = k;
      if (root.kind == NodeKind::Tuple) {
        for (int e : root.elems) res[k].push_back(mg.gen(e, fk));
      } else {
        res[k].push_back(mg.gen(ir.root, fk));
      }
    }
    mg.read_staged(staged);
    mg.emit(os, 4, opt.load_lookahead);
    fp64 |= mg.uses_fp64();
    return mg.vector_loads();
  };
  std::ostringstream multi;
  std::vector<std::vector<std::string>> mres;
  if (P > 1) merged_body(false, multi, mres);
  // The same with reads of a short innermost axis grouped into float4 loads
  // (cc_ew_vl / cc_sum_vl, launched when every input is 16-byte aligned).
  std::ostringstream vl_body;
  std::vector<std::vector<std::string>> vl_res;
  if (opt.vector_loads && !contiguous) g.has_vl = merged_body(true, vl_body, vl_res) > 0;
  // (cc_ew_vl reads the copies as float4: 16-byte aligned there)
  auto staging = [&](bool align16) {
    std::string code;
    for (auto &sp : staged) {
      const std::string k = std::to_string(sp.first), n = std::to_string(sp.second);
      code += std::string("  __shared__ ") + (align16 ? "__align__(16) " : "") + "float cc_sp" + k + "[" + n +
              "];\n  for (int i_ = threadIdx.x; i_ < " + n + "; i_ += blockDim.x) cc_sp" + k + "[i_] = __ldg(in" + k +
              " + i_);\n";
    }
    if (!code.empty()) code += "  __syncthreads();\n";
    return code;
  };
  const std::string stage_code = staging(false);
  g.uses_fp64_index = fp64;
  g.smem_bytes = ring_slots * opt.block * 4;
  const std::string ring_decl = ring_slots > 0 ? "  extern __shared__ float cc_ring[];\n" : "";

  std::string call_args;
  auto contig_call = [&](const std::string &lane) {
    std::string s = "cc_point(";
    for (int i = 0; i < ir.n_params; ++i) s += (i ? ", " : "") + std::string("v") + std::to_string(i) + lane;
    return s + ")";
  };

  // The float4 loop: each thread takes U float4 positions `stride` apart, loads
  // all of them from every input first (U * inputs loads in flight), then
  // computes; leftover positions and the last n % 4 floats follow one at a time.
  const int U = opt.vec_unroll > 0 ? opt.vec_unroll : 1;
  g.vec_unroll = U;
  auto vec4_loop = [&](int nin, int u_count, bool store, const std::function<std::string(const std::string &)> &call) {
    std::ostringstream o;
    o << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
      << "  const cc_i64 n4 = n >> 2;\n"
      << "  cc_i64 q = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x;\n"
      << "  for (; q + " << (u_count - 1) << " * stride < n4; q += " << u_count << " * stride) {\n";
    for (int u = 0; u < u_count; ++u)
      for (int i = 0; i < nin; ++i)
        o << "    const float4 v" << i << "_" << u << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q + "
          << u << " * stride);\n";
    if (store) o << "    cc_pdl_gate(cc_early);\n";
    for (int u = 0; u < u_count; ++u) {
      auto lane_call = [&](const char *lane) {
        std::string c = "cc_point(";
        for (int i = 0; i < nin; ++i) c += (i ? ", " : "") + std::string("v") + std::to_string(i) + "_" + std::to_string(u) + lane;
        return c + ")";
      };
      if (store) {
        o << "    {\n      float4 r;\n";
        for (const char *lane : {".x", ".y", ".z", ".w"}) o << "      r" << lane << " = " << lane_call(lane) << ";\n";
        o << "      reinterpret_cast<float4 *>(out)[q + " << u << " * stride] = r;\n    }\n";
      } else {
        for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    cc_acc(s_, c_, " << lane_call(lane) << ");\n";
      }
    }
    o << "  }\n  for (; q < n4; q += stride) {\n";
    for (int i = 0; i < nin; ++i)
      o << "    const float4 v" << i << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q);\n";
    if (store) {
      o << "    cc_pdl_gate(cc_early);\n    float4 r;\n";
      for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    r" << lane << " = " << call(lane) << ";\n";
      o << "    reinterpret_cast<float4 *>(out)[q] = r;\n";
    } else {
      for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    cc_acc(s_, c_, " << call(lane) << ");\n";
    }
    o << "  }\n  for (cc_i64 lin = (n4 << 2) + (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += stride) {\n";
    for (int i = 0; i < nin; ++i) o << "    const float v" << i << " = __ldg(in" << i << " + lin);\n";
    if (store)
      o << "    cc_pdl_gate(cc_early);\n    out[lin] = " << call("") << ";\n  }\n";
    else
      o << "    cc_acc(s_, c_, " << call("") << ");\n  }\n";
    return o.str();
  };

  // Scalar loads of the contiguous form: the kernel needs no shape, only n.
  std::string contig_scalar;
  if (contiguous) {
    for (int i = 0; i < ir.n_params; ++i)
      contig_scalar += "    const float v" + std::to_string(i) + " = __ldg(in" + std::to_string(i) + " + lin);\n";
  }
  if (ir.kind == ProgramKind::Elementwise && contiguous) {
    src << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_ew(" << params
        << "float *__restrict__ out, cc_i64 n) {\n"
        << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
        << "  for (cc_i64 lin = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += stride) {\n"
        << contig_scalar << "    cc_pdl_gate(cc_early);\n    out[lin] = " << contig_call("") << ";\n  }\n}\n\n"
        << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_ew_v4(" << params
        << "float *__restrict__ out, cc_i64 n) {\n"
        << vec4_loop(ir.n_params, U, true, contig_call) << "}\n\n";
  } else if (ir.kind == ProgramKind::Sum && contiguous) {
    src << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_sum(" << params
        << "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out, cc_i64 n) {\n"
        << "  float s_ = 0.0f, c_ = 0.0f;\n"
        << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
        << "  for (cc_i64 lin = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += stride) {\n"
        << contig_scalar << "    cc_acc(s_, c_, " << contig_call("") << ");\n  }\n"
        << "  cc_grid_finish_pdl(s_, c_, partials, counter, out, cc_early);\n}\n\n"
        << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_sum_v4(" << params
        << "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out, cc_i64 n) {\n"
        << "  float s_ = 0.0f, c_ = 0.0f;\n"
        << vec4_loop(ir.n_params, U, false, contig_call)
        << "  cc_grid_finish_pdl(s_, c_, partials, counter, out, cc_early);\n}\n\n";
  } else if (ir.kind == ProgramKind::Elementwise) {
    auto ew_kernel = [&](const std::string &name, const std::string &ring, const std::string &body,
                         const std::vector<std::vector<std::string>> &point_results) {
      src << "extern \"C\" __global__ void __launch_bounds__(" << lb << ") " << name << "(" << params
          << "float *__restrict__ out, cc_i64 n) {\n" << ring << (name == "cc_ew_vl" ? staging(true) : stage_code)
          << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
          << (P > 1 ? "  for (cc_i64 lin = ((cc_i64)blockIdx.x * blockDim.x + threadIdx.x) * " + std::to_string(P) +
                          "; lin < n; lin += stride * " + std::to_string(P) + ") {\n"
                    : std::string("  for (cc_i64 lin = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += "
                                  "stride) {\n"))
          << body;
      src << "    cc_pdl_gate(cc_early);\n";
      // point `p` of this thread (p = 0 .. P-1) stores `res`
      auto store = [&](const std::string &p, const std::vector<std::string> &res) {
        const std::string at = p == "0" ? std::string("lin") : "(lin + " + p + ")";
        if (g.tuple_len == 1) {
          src << "    out[" << at << "] = " << res[0] << ";\n";
        } else if (g.tuple_len % 4 == 0) {
          // a point's tuple is tuple_len consecutive floats: float4 stores when aligned
          src << "    if ((reinterpret_cast<unsigned long long>(out) & 15ull) == 0) {\n"
              << "      float4 *o4_ = reinterpret_cast<float4 *>(out + " << at << " * " << g.tuple_len << "LL);\n";
          for (int k = 0; k < g.tuple_len; k += 4)
            src << "      o4_[" << k / 4 << "] = make_float4(" << res[k] << ", " << res[k + 1] << ", " << res[k + 2]
                << ", " << res[k + 3] << ");\n";
          src << "    } else {\n";
          for (int k = 0; k < g.tuple_len; ++k)
            src << "      out[" << at << " * " << g.tuple_len << "LL + " << k << "] = " << res[k] << ";\n";
          src << "    }\n";
        } else {
          for (int k = 0; k < g.tuple_len; ++k)
            src << "    out[" << at << " * " << g.tuple_len << "LL + " << k << "] = " << res[k] << ";\n";
        }
      };
      for (int k = 0; k < P; ++k) store(std::to_string(k), point_results[k]);
      src << "  }\n}\n\n";
    };
    if (P > 1)
      ew_kernel("cc_ew", ring_decl, multi.str(), mres);
    else
      ew_kernel("cc_ew", ring_decl, generic.str(), {results});
    if (g.has_vl) ew_kernel("cc_ew_vl", "", vl_body.str(), vl_res);
    if (contiguous) {
      src << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_ew_v4(" << params
          << "float *__restrict__ out, cc_i64 n) {\n"
          << vec4_loop(ir.n_params, U, true, contig_call) << "}\n\n";
    }
  } else {
    src << "extern \"C\" __global__ void __launch_bounds__(" << lb << ") cc_sum(" << params
        << "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out, cc_i64 n) {\n"
        << ring_decl << stage_code << "  float s_ = 0.0f, c_ = 0.0f;\n"
        << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
        << "  for (cc_i64 lin = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += stride) {\n"
        << generic.str() << "    cc_acc(s_, c_, " << results[0] << ");\n  }\n"
        << "  cc_grid_finish_pdl(s_, c_, partials, counter, out, cc_early);\n}\n\n";
    if (g.has_vl) {
      // the same points in the same order: only the reads differ, so the sum's bits do not
      src << "extern \"C\" __global__ void __launch_bounds__(" << lb << ") cc_sum_vl(" << params
          << "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out, cc_i64 n) {\n"
          << staging(true) << "  float s_ = 0.0f, c_ = 0.0f;\n"
          << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
          << "  for (cc_i64 lin = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x; lin < n; lin += stride) {\n"
          << vl_body.str() << "    cc_acc(s_, c_, " << vl_res[0][0] << ");\n  }\n"
          << "  cc_grid_finish_pdl(s_, c_, partials, counter, out, cc_early);\n}\n\n";
    }
    if (contiguous) {
      src << "extern \"C\" __global__ void __launch_bounds__(" << block << ") cc_sum_v4(" << params
          << "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out, cc_i64 n) {\n"
          << "  float s_ = 0.0f, c_ = 0.0f;\n"
          << vec4_loop(ir.n_params, U, false, contig_call)
          << "  cc_grid_finish_pdl(s_, c_, partials, counter, out, cc_early);\n}\n\n";
    }
  }
  g.source = src.str();
  // every kernel orders itself after the kernels it depends on (cc_pdl_begin / cc_pdl_gate)
  const std::string sig_end = ", cc_i64 n) {\n";
  const std::string with_flag = ", cc_i64 n, int cc_early) {\n  cc_pdl_begin(cc_early);\n";
  for (size_t at = g.source.find(sig_end); at != std::string::npos; at = g.source.find(sig_end, at)) {
    g.source.replace(at, sig_end.size(), with_flag);
    at += with_flag.size();
  }
  return g;
}

}  // namespace cc

// ---------------------------------------------------------------- tunable form

namespace cc {

bool is_tunable(const Ir &ir, std::string *why) {
  auto no = [&](const char *w) {
    if (why) *why = w;
    return false;
  };
  if (ir.nodes[ir.root].kind == NodeKind::Tuple) return no("a tuned program has one value per point (no join)");
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  if (domain <= 0) return no("a tuned program has at least one point");
  // The cost model knows programs of up to 47 nodes (its training workloads);
  // larger ones run their standard kernel (their six-kernel tunable form also
  // compiles slowly: over a minute for the 262-node view-heavy op).
  if ((int)ir.nodes.size() > kTuneMaxNodes) return no("a tuned program has at most 64 nodes");
  return true;
}

std::string tunable_source(const Ir &ir, const std::string &suffix) {
  const bool contiguous = program_is_contiguous(ir);
  const bool sum = ir.kind == ProgramKind::Sum;
  const int nin = ir.n_params;
  const int rank = (int)ir.out_shape.size();
  std::ostringstream o;
  const std::string P = (contiguous ? "cc_pt" : "cc_gp") + suffix;
  Frame f0{0, {}, ir.out_shape};
  if (contiguous) {
    Generator gen(ir, true);
    std::ostringstream body;
    std::string r = gen.gen(ir.root, f0);
    gen.emit(body, 2, 0);
    o << "static __device__ __forceinline__ float " << P << "(";
    for (int i = 0; i < nin; ++i) o << (i ? ", " : "") << "float a" << i;
    if (nin == 0) o << "void";
    o << ") {\n" << body.str() << "  return " << r << ";\n}\n";
  } else {
    // The generic point: output coordinates decoded from `lin`, then the
    // program's loads and arithmetic.
    for (int d = 0; d < rank; ++d) f0.gid.push_back("g" + std::to_string(d));
    Generator gen(ir, false, true, -1);
    std::ostringstream body;
    int64_t domain = 1;
    for (int64_t d : ir.out_shape) domain *= d;
    if (rank > 0) body << decode_coordinates(ir.out_shape, domain, "  ");
    std::string r = gen.gen(ir.root, f0);
    gen.emit(body, 2, 8);
    o << "static __device__ __forceinline__ float " << P << "(cc_i64 lin";
    for (int i = 0; i < nin; ++i) o << ", const float *__restrict__ in" << i;
    o << ") {\n" << body.str() << "  return " << r << ";\n}\n";
  }
  std::string params;
  for (int i = 0; i < nin; ++i) params += "const float *__restrict__ in" + std::to_string(i) + ", ";
  std::string ins;
  for (int i = 0; i < nin; ++i) ins += ", in" + std::to_string(i);
  // value at scalar position `pos` (an expression of type cc_i64)
  auto scalar_value = [&](const std::string &pos, std::ostringstream &os, const std::string &var,
                          const std::string &pad) {
    if (contiguous) {
      for (int i = 0; i < nin; ++i)
        os << pad << "const float " << var << "_a" << i << " = __ldg(in" << i << " + " << pos << ");\n";
      os << pad << "const float " << var << " = " << P << "(";
      for (int i = 0; i < nin; ++i) os << (i ? ", " : "") << var << "_a" << i;
      os << ");\n";
    } else {
      os << pad << "const float " << var << " = " << P << "(" << pos << ins << ");\n";
    }
  };
  auto consume = [&](const std::string &pos, const std::string &val) {
    return sum ? "cc_acc(s_, c_, " + val + ");" : "out[" + pos + "] = " + val + ";";
  };
  for (int V : {1, 4}) {
    for (int E : {1, 2, 4}) {
      o << "extern \"C\" __global__ void __launch_bounds__(512) cc_t" << suffix << "_v" << V << "_e" << E << "("
        << params
        << (sum ? "float2 *__restrict__ partials, unsigned int *__restrict__ counter, float *__restrict__ out"
                : "float *__restrict__ out")
        << ", cc_i64 n) {\n";
      // launched with programmatic dependent launch: wait for the previous kernel
      // before any memory access (a no-op without the launch attribute)
      o << "  cc_pdl_wait_then_release();\n";
      if (sum) o << "  float s_ = 0.0f, c_ = 0.0f;\n";
      o << "  const cc_i64 stride = (cc_i64)gridDim.x * blockDim.x;\n"
        << "  const cc_i64 tid = (cc_i64)blockIdx.x * blockDim.x + threadIdx.x;\n";
      if (V == 1) {
        o << "  cc_i64 lin = tid;\n  for (; lin + " << (E - 1) << " * stride < n; lin += " << E << " * stride) {\n";
        if (contiguous) {
          // every load of the E positions first, then the arithmetic
          for (int e = 0; e < E; ++e)
            for (int i = 0; i < nin; ++i)
              o << "    const float x" << e << "_" << i << " = __ldg(in" << i << " + lin + " << e << " * stride);\n";
          for (int e = 0; e < E; ++e) {
            std::string call = P + "(";
            for (int i = 0; i < nin; ++i) call += (i ? ", " : "") + std::string("x") + std::to_string(e) + "_" + std::to_string(i);
            call += ")";
            o << "    " << consume("lin + " + std::to_string(e) + " * stride", call) << "\n";
          }
        } else {
          for (int e = 0; e < E; ++e)
            o << "    const float r" << e << " = " << P << "(lin + " << e << " * stride" << ins << ");\n";
          for (int e = 0; e < E; ++e)
            o << "    " << consume("lin + " + std::to_string(e) + " * stride", "r" + std::to_string(e)) << "\n";
        }
        o << "  }\n  for (; lin < n; lin += stride) {\n";
        scalar_value("lin", o, "r", "    ");
        o << "    " << consume("lin", "r") << "\n  }\n";
      } else if (contiguous) {
        // float4 loads: E float4 positions `stride` apart per thread
        o << "  const cc_i64 n4 = n >> 2;\n  cc_i64 q = tid;\n"
          << "  for (; q + " << (E - 1) << " * stride < n4; q += " << E << " * stride) {\n";
        for (int e = 0; e < E; ++e)
          for (int i = 0; i < nin; ++i)
            o << "    const float4 x" << e << "_" << i << " = __ldg(reinterpret_cast<const float4 *>(in" << i
              << ") + q + " << e << " * stride);\n";
        for (int e = 0; e < E; ++e) {
          auto lane_call = [&](const char *lane) {
            std::string c = P + "(";
            for (int i = 0; i < nin; ++i) c += (i ? ", " : "") + std::string("x") + std::to_string(e) + "_" + std::to_string(i) + lane;
            return c + ")";
          };
          if (sum) {
            for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    cc_acc(s_, c_, " << lane_call(lane) << ");\n";
          } else {
            o << "    {\n      float4 r;\n";
            for (const char *lane : {".x", ".y", ".z", ".w"}) o << "      r" << lane << " = " << lane_call(lane) << ";\n";
            o << "      reinterpret_cast<float4 *>(out)[q + " << e << " * stride] = r;\n    }\n";
          }
        }
        o << "  }\n  for (; q < n4; q += stride) {\n";
        for (int i = 0; i < nin; ++i)
          o << "    const float4 x_" << i << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q);\n";
        auto lane_call = [&](const char *lane) {
          std::string c = P + "(";
          for (int i = 0; i < nin; ++i) c += (i ? ", " : "") + std::string("x_") + std::to_string(i) + lane;
          return c + ")";
        };
        if (sum) {
          for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    cc_acc(s_, c_, " << lane_call(lane) << ");\n";
        } else {
          o << "    float4 r;\n";
          for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    r" << lane << " = " << lane_call(lane) << ";\n";
          o << "    reinterpret_cast<float4 *>(out)[q] = r;\n";
        }
        o << "  }\n  for (cc_i64 lin = (n4 << 2) + tid; lin < n; lin += stride) {\n";
        scalar_value("lin", o, "r", "    ");
        o << "    " << consume("lin", "r") << "\n  }\n";
      } else {
        // four consecutive points per work item, one float4 store when whole
        o << "  const cc_i64 nw = (n + 3) >> 2;\n  cc_i64 w = tid;\n"
          << "  for (; w + " << (E - 1) << " * stride < nw; w += " << E << " * stride) {\n";
        for (int e = 0; e < E; ++e) {
          const std::string b = "b" + std::to_string(e);
          o << "    const cc_i64 " << b << " = (w + " << e << " * stride) << 2;\n"
            << "    if (" << b << " + 3 < n) {\n";
          for (int v = 0; v < 4; ++v)
            o << "      const float r" << v << " = " << P << "(" << b << " + " << v << ins << ");\n";
          if (sum)
            o << "      cc_acc(s_, c_, r0);\n      cc_acc(s_, c_, r1);\n      cc_acc(s_, c_, r2);\n      cc_acc(s_, c_, r3);\n";
          else
            o << "      reinterpret_cast<float4 *>(out)[" << b << " >> 2] = make_float4(r0, r1, r2, r3);\n";
          o << "    } else {\n      for (cc_i64 lin = " << b << "; lin < n; ++lin) {\n";
          scalar_value("lin", o, "r", "        ");
          o << "        " << consume("lin", "r") << "\n      }\n    }\n";
        }
        o << "  }\n  for (; w < nw; w += stride) {\n"
          << "    for (cc_i64 lin = w << 2; lin < n && lin < (w << 2) + 4; ++lin) {\n";
        scalar_value("lin", o, "r", "      ");
        o << "      " << consume("lin", "r") << "\n    }\n  }\n";
      }
      if (sum) o << "  cc_grid_finish(s_, c_, partials, counter, out);\n";
      o << "}\n";
    }
  }
  return o.str();
}

}  // namespace cc

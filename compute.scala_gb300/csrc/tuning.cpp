// The tuner's configuration space and the cost model's features of a program.
//
// The reference leaves the launch shape to the OpenCL runtime
// (Tensors.scala:1360-1375 passes no local size; reductions take
// min(length, CL_KERNEL_WORK_GROUP_SIZE), Tensors.scala:700); here every
// program can be run in 48 launch configurations and the tuner picks one.
#include <cmath>
#include <cstring>

#include "internal.h"
#include "kernels.h"

namespace cc {

TuneConfig tune_config(int index) {
  static const int blocks[4] = {64, 128, 256, 512};
  static const int epts[3] = {1, 2, 4};
  TuneConfig c;
  c.block = blocks[index % 4];
  c.vec = (index / 4) % 2 ? 4 : 1;
  c.ept = epts[(index / 8) % 3];
  c.split = (index / 24) % 2 ? 2 : 1;
  return c;
}

int tune_kernel_index(const TuneConfig &c) { return (c.vec == 4 ? 3 : 0) + (c.ept == 1 ? 0 : c.ept == 2 ? 1 : 2); }

int64_t tune_grid(int64_t n, const TuneConfig &c, bool sum, int sm_count, int resident) {
  const int64_t items = c.vec == 4 ? (n + 3) / 4 : n;
  const int64_t threads = (items + c.ept - 1) / c.ept;
  int64_t grid = (threads + c.block - 1) / c.block;
  if (c.split == 1) {
    const int64_t wave = (int64_t)sm_count * (resident > 0 ? resident : 1);
    if (grid > wave) grid = wave;
  }
  if (sum && grid > kMaxSumBlocks) grid = kMaxSumBlocks;
  if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
  return grid < 1 ? 1 : grid;
}

namespace {

float lg(double x) { return (float)std::log2(1.0 + x); }

}  // namespace

void program_features(const Ir &ir, int config, int sm_count, float *f) {
  std::memset(f, 0, sizeof(float) * kFeatures);
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  const bool sum = ir.kind == ProgramKind::Sum;
  f[0] = sum ? 1.0f : 0.0f;
  f[1] = lg((double)domain);
  f[2] = (float)ir.out_shape.size();
  for (size_t d = 0; d < ir.out_shape.size() && d < 4; ++d) f[3 + d] = lg((double)ir.out_shape[d]);
  f[7] = (float)ir.n_params;
  double param_elems = 0;
  int views = 0, extracts = 0, literals = 0, ops = 0, transcendental = 0, bounded = 0;
  int unit_inner = 0, zero_inner = 0, other_inner = 0;
  bool fractional = false;
  for (const IrNode &n : ir.nodes) {
    switch (n.kind) {
      case NodeKind::Param: {
        double e = 1;
        for (int64_t d : n.dims) e *= (double)d;
        param_elems += e;
        break;
      }
      case NodeKind::Literal: ++literals; break;
      case NodeKind::View:
      case NodeKind::Extract: {
        if (n.kind == NodeKind::View) ++views; else ++extracts;
        const std::vector<int64_t> &dims = n.kind == NodeKind::View ? n.dims : ir.nodes[n.a].dims;
        const int rows = (int)dims.size();
        bool any_bound = false;
        for (int y = 0; y < rows; ++y) {
          bool nonzero = false;
          for (int x = 0; x < n.cols; ++x) {
            const double s = n.m[(size_t)y * n.cols + x];
            if (s != 0.0) nonzero = true;
            if (s != std::floor(s)) fractional = true;
          }
          any_bound |= nonzero;
        }
        if (any_bound && !(n.kind == NodeKind::Extract && rows == (int)ir.out_shape.size())) ++bounded;
        if (n.kind == NodeKind::Extract) {
          const double inner = (rows > 0 && n.cols >= 2) ? n.m[(size_t)(rows - 1) * n.cols + (n.cols - 2)] : 0.0;
          if (inner == 1.0) ++unit_inner; else if (inner == 0.0) ++zero_inner; else ++other_inner;
        }
        break;
      }
      case NodeKind::Unary:
        ++ops;
        f[13 + n.op] += 1.0f;  // neg exp log tanh abs sqrt: 13..18
        if (n.op == (uint8_t)UnOp::Exp || n.op == (uint8_t)UnOp::Log || n.op == (uint8_t)UnOp::Tanh) ++transcendental;
        break;
      case NodeKind::Binary:
        ++ops;
        f[19 + n.op] += 1.0f;  // + - * / % min max: 19..25
        break;
      case NodeKind::Tuple: break;
    }
  }
  const bool contiguous = !contiguous_structure_key(ir).empty();
  f[8] = lg(param_elems);
  f[9] = contiguous ? 1.0f : 0.0f;
  f[10] = (float)views;
  f[11] = (float)extracts;
  f[12] = (float)literals;
  f[26] = (float)ops;
  f[27] = (float)transcendental;
  f[28] = (float)bounded;
  f[29] = (float)unit_inner;
  f[30] = (float)zero_inner;
  f[31] = (float)other_inner;
  f[32] = fractional ? 1.0f : 0.0f;
  const double bytes = 4.0 * (std::min(param_elems, (double)domain * ir.n_params) + (sum ? 1.0 : (double)domain));
  f[33] = lg(bytes);
  f[34] = (float)ops / (float)(extracts + 1);
  f[35] = domain % 4 == 0 ? 1.0f : 0.0f;
  f[36] = ir.out_shape.empty() ? 0.0f : lg((double)ir.out_shape.back());
  f[37] = lg((double)domain / (double)(sm_count > 0 ? sm_count : 1) / 2048.0);
  // the configuration
  const TuneConfig c = tune_config(config);
  f[44 + (config % 4)] = 1.0f;
  f[48 + (c.vec == 4 ? 1 : 0)] = 1.0f;
  f[50 + (c.ept == 1 ? 0 : c.ept == 2 ? 1 : 2)] = 1.0f;
  f[53 + (c.split == 2 ? 1 : 0)] = 1.0f;
  f[55] = (float)std::log2((double)c.block);
  int resident = 2048 / c.block;
  if (resident > 32) resident = 32;
  const int64_t grid = tune_grid(domain, c, sum, sm_count, resident);
  f[56] = lg((double)grid);
  f[57] = lg((double)grid * c.block);
  f[58] = lg((double)grid / ((double)(sm_count > 0 ? sm_count : 1) * resident));
  f[59] = lg((double)domain / ((double)grid * c.block));
  f[60] = (c.vec == 4 && contiguous) ? 1.0f : 0.0f;
  f[61] = (c.vec == 4 && !contiguous) ? 1.0f : 0.0f;
  f[62] = (sum && c.split == 2) ? 1.0f : 0.0f;
  f[63] = 1.0f;
}

}  // namespace cc

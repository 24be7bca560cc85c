// EvaluateCircuit on the GPU (the flow of src/evaluate_circuit.cpp:106-253):
// parse -> output states -> network description -> static program ->
// one batched replay per group of final states.
#include "engine.h"

#include "tc_gemm.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

namespace qfx {

std::string cuda_error_string(cudaError_t e, const char* what) {
  return cat("ERROR (qflex_gb300: CUDA ", what, ") --> ", cudaGetErrorString(e));
}

#define QFX_CUDA(call)                                                  \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) throw cuda_error_string(e_, #call);          \
  } while (0)

// Identifies the buffers a captured device pass was recorded with.
struct GraphKey {
  int batch = 0;
  const void* arena = nullptr;
  const void* ws = nullptr;
  const void* bits = nullptr;
  const void* amps = nullptr;
  unsigned options = 0;
  int precision = -1;
  bool operator==(const GraphKey& o) const {
    return batch == o.batch && arena == o.arena && ws == o.ws && bits == o.bits && amps == o.amps &&
           options == o.options && precision == o.precision;
  }
};

struct Engine::Plan {
  std::string key;
  Circuit circuit;
  Grid grid;
  Ordering ordering;
  std::vector<Op> ops;
  bool built = false;
  Network net;
  Program prog;
  std::vector<PermPlan> perm;  // indexed like prog.ops (unused for GEMM ops)
  // 3xFP16 fusion, indexed like prog.ops: a permute that writes the next
  // product's A operand straight as FP16 planes has fused[i] = index of that
  // product; the product has fused[j] = j. -1 elsewhere. Recomputed when
  // the options change (fuse_version).
  std::vector<int> fused;
  unsigned fuse_version = ~0u;
  int precision = -1;          // precision the program was planned for
  std::size_t tc_ws_elems = 0; // split-plane workspace of one batch entry
  std::uint32_t max_size_log2 = 0;
  ColumnDesc* d_cols = nullptr;
  StepDesc* d_steps = nullptr;
  float2* d_mats = nullptr;
  float2* d_mats_lo = nullptr;  // null: plain FP32 columns
  double2* d_mats64 = nullptr;  // complex128 programs: the double gate data
  std::uint32_t* d_ptr = nullptr;
  std::uint32_t* d_leaves = nullptr;
  // Captured device pass and the buffers it was captured with.
  cudaGraphExec_t graph = nullptr;
  GraphKey graph_key, seen_key;
  std::size_t graph_launches = 0;
  ~Plan() {
    if (graph) cudaGraphExecDestroy(graph);
    cudaFree(d_cols);
    cudaFree(d_steps);
    cudaFree(d_mats);
    cudaFree(d_mats_lo);
    cudaFree(d_mats64);
    cudaFree(d_ptr);
    cudaFree(d_leaves);
  }
};

Engine::Engine(int device, int precision) : device_(device), precision_(precision), tc_cfg_(tc_default_config()) {
  if (device < 0) {  // planning only: no CUDA calls at all
    set_precision(precision);
    return;
  }
  int n = 0;
  QFX_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) throw QFX_ERR("CUDA device ", device, " does not exist (", n, " visible).");
  QFX_CUDA(cudaSetDevice(device_));
  QFX_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  own_stream_ = true;
  if (const char* g = std::getenv("QFLEX_GB300_GRAPHS")) graphs_ = std::atoi(g) != 0;
  if (const char* f = std::getenv("QFLEX_GB300_FUSE")) fuse_splits_ = std::atoi(f) != 0;
  QFX_CUDA(cudaEventCreate(&ev0_));
  QFX_CUDA(cudaEventCreate(&ev1_));
  set_precision(precision);
}

Engine::~Engine() {
  if (device_ < 0) return;
  cudaSetDevice(device_);
  if (stream_) cudaStreamSynchronize(stream_);
  plan_.reset();
  for (auto& b : bufs_) cudaFree(b.ptr);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  for (auto e : prof_events_) cudaEventDestroy(e);
  if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

void Engine::set_precision(int p) {
  if (p != FP32 && p != TF32X3 && p != FP16X3 && p != BF16X3 && p != FP64 && p != FP64_FF)
    throw QFX_ERR("Precision mode ", p, " is not available in this build.");
  precision_ = p;
}

void Engine::set_option(const std::string& name, double value) {
  if (name == "tc_chunk") {
    if (!(value >= 1 && value <= 64) || value != double(int(value)))
      throw QFX_ERR("Option tc_chunk must be an integer in 1..64.");
    tc_cfg_.chunk = int(value);
  } else if (name == "tc_variant") {
    if (!(value >= 0 && value <= 4) || value != double(int(value)))
      throw QFX_ERR("Option tc_variant must be 0, 1, 2, 3 or 4.");
    tc_cfg_.variant = int(value);
  } else if (name == "tc_pair") {
    if (value != 0 && value != 1) throw QFX_ERR("Option tc_pair must be 0 or 1.");
    tc_cfg_.variant = value == 0 ? 0 : -1;
  } else if (name == "graphs") {
    if (value != 0 && value != 1) throw QFX_ERR("Option graphs must be 0 or 1.");
    graphs_ = value != 0;
  } else if (name == "fuse_splits") {
    if (value != 0 && value != 1) throw QFX_ERR("Option fuse_splits must be 0 or 1.");
    fuse_splits_ = value != 0;
  } else if (name == "open_terminals") {
    if (value != 0 && value != 1) throw QFX_ERR("Option open_terminals must be 0 or 1.");
    open_terminals_ = value != 0;
  } else if (name == "tc_debias") {
    if (value != 0 && value != 1) throw QFX_ERR("Option tc_debias must be 0 or 1.");
    debias_ = value != 0;
    if (device_ >= 0) {
      const int flag = debias_ ? 1 : 0;
      int* p = error_flag();
      QFX_CUDA(cudaMemcpyAsync(p + 1, &flag, sizeof(flag), cudaMemcpyHostToDevice, stream_));
      QFX_CUDA(cudaStreamSynchronize(stream_));
    }
  } else if (name == "exact_gates") {
    if (value != -1 && value != 0 && value != 1) throw QFX_ERR("Option exact_gates must be -1, 0 or 1.");
    exact_gates_ = int(value);
  } else if (name == "tc_wait_ns") {
    if (!(value >= 0 && value <= 1e11) || value != double((unsigned long long)value))
      throw QFX_ERR("Option tc_wait_ns must be an integer in 0..1e11.");
    wait_ns_ = (unsigned long long)value;
    if (device_ >= 0) {
      int* p = error_flag();
      QFX_CUDA(cudaMemcpyAsync(p + 2, &wait_ns_, sizeof(wait_ns_), cudaMemcpyHostToDevice, stream_));
      QFX_CUDA(cudaStreamSynchronize(stream_));
    }
  } else if (name == "max_batch") {
    if (!(value >= 0 && value <= 65535) || value != double(int(value)))
      throw QFX_ERR("Option max_batch must be an integer in 0..65535.");
    max_batch_ = int(value);
  } else {
    throw QFX_ERR("Unknown option '", name, "'.");
  }
  ++options_version_;
}

double Engine::get_option(const std::string& name) const {
  if (name == "tc_chunk") return tc_cfg_.chunk;
  if (name == "tc_pair") return tc_cfg_.variant == 0 ? 0 : 1;
  if (name == "tc_variant") return tc_cfg_.variant;
  if (name == "graphs") return graphs_ ? 1 : 0;
  if (name == "max_batch") return max_batch_;
  if (name == "open_terminals") return open_terminals_ ? 1 : 0;
  if (name == "fuse_splits") return fuse_splits_ ? 1 : 0;
  if (name == "tc_wait_ns") return double(wait_ns_);
  if (name == "exact_gates") return exact_gates_;
  if (name == "tc_debias") return debias_ ? 1 : 0;
  throw QFX_ERR("Unknown option '", name, "'.");
}

void Engine::set_tc_variant(std::size_t m, std::size_t n, std::size_t k, int variant) {
  if (variant < -1 || variant > 4) throw QFX_ERR("Tensor-core variant must be -1, 0, 1, 2, 3 or 4.");
  if (variant == -1)
    tc_variant_.erase({m, n, k});
  else
    tc_variant_[{m, n, k}] = variant;
  ++options_version_;
}

void Engine::launch_split_product(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                                  std::size_t k, std::uint64_t ac_stride, std::uint64_t bt_stride, int batch,
                                  float* ws) {
  const TcConfig cfg = tc_config(m, n, k);
  if (precision_ == FP16X3)
    launch_cgemm_fp16x3(A, Bt, C, m, n, k, ac_stride, bt_stride, batch, ws, error_flag(), cfg, stream_);
  else if (precision_ == BF16X3)
    launch_cgemm_bf16x3(A, Bt, C, m, n, k, ac_stride, bt_stride, batch, ws, error_flag(), cfg, stream_);
  else
    launch_cgemm_tf32x3(A, Bt, C, m, n, k, ac_stride, bt_stride, batch, ws, error_flag(), cfg, stream_);
}

TcConfig Engine::tc_config(std::size_t m, std::size_t n, std::size_t k) const {
  TcConfig c = tc_cfg_;
  const auto it = tc_variant_.find({m, n, k});
  if (it != tc_variant_.end()) c.variant = it->second;
  return c;
}

int* Engine::error_flag() {
  // The context's control block for the tensor-core kernels, int[4]: the
  // error code they set, the truncation-bias compensation switch, then
  // (bytes 8..15) the limit of their pipeline waits in ns (0: 2 s).
  const bool fresh = (int)bufs_.size() <= 5 || bufs_[5].bytes < 4 * sizeof(int);
  int* p = (int*)reserve(sizeof(int) * 4, 5);
  if (fresh) {
    int init[4] = {0, debias_ ? 1 : 0, 0, 0};
    std::memcpy(init + 2, &wait_ns_, sizeof(wait_ns_));
    QFX_CUDA(cudaMemcpyAsync(p, init, sizeof(init), cudaMemcpyHostToDevice, stream_));
    QFX_CUDA(cudaStreamSynchronize(stream_));
  }
  return p;
}

float* Engine::tc_workspace(std::size_t elems) {
  return (float*)reserve(std::max<std::size_t>(elems, 1) * sizeof(float), 4);
}

void Engine::check_error_flag() {
  int h = 0;
  QFX_CUDA(cudaMemcpyAsync(&h, error_flag(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
  QFX_CUDA(cudaStreamSynchronize(stream_));
  if (h != 0) {
    QFX_CUDA(cudaMemsetAsync(error_flag(), 0, sizeof(int), stream_));
    throw cat("ERROR (qflex_gb300: CUDA tensor-core pipeline) --> A tensor-core pipeline wait expired (code ", h,
              "); results discarded.");
  }
}

void Engine::multiply(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                      std::size_t k, std::uint64_t stride, int batch) {
  if (is_complex128(precision_))
    throw QFX_ERR("The complex64 tensor operations need a complex64 precision mode (this context is complex128).");
  if (precision_ != FP32 && tc_eligible(m, n, k)) {
    // The tensor-core kernel reads B as [n][k]: transpose into the front of
    // the workspace, split planes after it.
    const std::size_t bt = ((n * k * (std::size_t)batch + 63) / 64) * 64;
    float* ws = tc_workspace(2 * bt + tc_workspace_elems(m, n, k) * (std::size_t)batch);
    float2* Bt = reinterpret_cast<float2*>(ws);
    int nbits = 0;
    std::uint8_t perm[40] = {};
    int ln = 0, lk = 0;
    while ((std::size_t(1) << ln) < n) ++ln;
    while ((std::size_t(1) << lk) < k) ++lk;
    if ((std::size_t(1) << ln) == n && (std::size_t(1) << lk) == k) {
      nbits = ln + lk;
      for (int b = 0; b < ln; ++b) perm[b] = (std::uint8_t)(lk + b);   // n digits move up
      for (int b = 0; b < lk; ++b) perm[ln + b] = (std::uint8_t)b;     // k digits move down
      PermPlan plan;
      make_perm_plan(nbits, perm, &plan);
      for (int b = 0; b < batch; ++b)
        launch_permute(plan, B + (std::size_t)b * stride, Bt + (std::size_t)b * n * k, 0, 1, stream_);
      launch_split_product(A, Bt, C, m, n, k, stride, n * k, batch, ws + 2 * bt);
      return;
    }
  }
  launch_cgemm_fp32(A, B, C, m, n, k, stride, batch, stream_, skinny_scratch());
}

void Engine::set_stream(cudaStream_t s) {
  if (own_stream_ && stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
  own_stream_ = false;
  stream_ = s;
}

void* Engine::reserve(std::size_t bytes, int slot) {
  if ((int)bufs_.size() <= slot) bufs_.resize(slot + 1);
  DevBuf& b = bufs_[slot];
  if (b.bytes < bytes) {
    QFX_CUDA(cudaStreamSynchronize(stream_));
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    QFX_CUDA(cudaMalloc(&b.ptr, bytes));
    b.bytes = bytes;
  }
  return b.ptr;
}

const std::vector<GemmShape>& Engine::last_shapes() const {
  static const std::vector<GemmShape> none;
  return plan_ && plan_->built ? plan_->prog.shapes : none;
}

const Program* Engine::last_program() const {
  return plan_ && plan_->built ? &plan_->prog : nullptr;
}

Engine::Plan* Engine::get_plan(const std::string& circuit, const std::string& ordering,
                               const std::string& grid) {
  std::string key = circuit;
  key += '\x01';
  key += ordering;
  key += '\x01';
  key += grid;
  key += '\x01';
  key += std::to_string(precision_);
  key += open_terminals_ ? "o" : "p";
  key += std::to_string(exact_gates_);
  if (plan_ && plan_->key == key) return plan_.get();
  auto p = std::make_unique<Plan>();
  p->key = std::move(key);
  p->grid.load(grid);
  p->circuit.load(circuit);
  p->ordering.load(ordering);
  p->ops = parse_ordering(p->ordering, p->grid);
  plan_ = std::move(p);
  return plan_.get();
}

namespace {

// Flatten descriptors: where each column's 2D tensor lives and which bit of
// its element index each two-qubit half reads.
void build_flatten_tables(const Network& net, const Program& prog, bool exact_gates,
                          std::vector<ColumnDesc>* cols, std::vector<StepDesc>* steps,
                          std::vector<float2>* mats, std::vector<float2>* mats_lo,
                          std::vector<double2>* mats64, std::uint32_t* max_log2) {
  *max_log2 = 0;
  for (std::size_t c = 0; c < net.columns.size(); ++c) {
    const QubitColumn& col = net.columns[c];
    const std::size_t r = col.indices.size();
    std::vector<int> lg(r), start(r, 0);
    int total = 0;
    for (std::size_t i = 0; i < r; ++i) {
      int l = 0;
      while ((std::size_t(1) << l) < col.dims[i]) ++l;
      lg[i] = l;
      total += l;
    }
    for (std::size_t i = r; i-- > 1;) start[i - 1] = start[i] + lg[i];
    ColumnDesc cd{};
    cd.out_offset = prog.column_offset[c];
    cd.size_log2 = (std::uint32_t)total;
    cd.step_begin = (std::uint32_t)steps->size();
    cd.o_shift = col.terminal ? start[0] : -1;
    *max_log2 = std::max(*max_log2, cd.size_log2);
    for (const ColumnStep& s : col.steps) {
      StepDesc sd{};
      sd.kind = (std::uint32_t)s.kind;
      sd.V = (std::uint32_t)s.V;
      sd.mat = (std::uint32_t)(mats64 ? mats64->size() : mats->size());
      if (s.kind == 2) {
        const Link& L = net.links[s.link];
        auto it = std::find(col.indices.begin(), col.indices.end(), L.name);
        if (it == col.indices.end()) throw QFX_ERR("Bond ", L.name, " is missing from its tensor.");
        int shift = start[it - col.indices.begin()];
        for (int u = s.ordinal + 1; u < L.n_gates; ++u) {
          int l = 0;
          while ((1 << l) < L.V[u]) ++l;
          shift += l;
        }
        sd.shift = (std::uint32_t)shift;
      }
      if (mats64) {
        for (const auto& z : s.exact) mats64->push_back(make_double2(z.real(), z.imag()));
      } else if (exact_gates) {
        // hi + lo of each double-precision constant
        for (const auto& z : s.exact) {
          const float hr = float(z.real()), hi = float(z.imag());
          mats->push_back(make_float2(hr, hi));
          mats_lo->push_back(make_float2(float(z.real() - double(hr)), float(z.imag() - double(hi))));
        }
      } else {
        for (const auto& z : s.data) mats->push_back(make_float2(z.real(), z.imag()));
      }
      steps->push_back(sd);
    }
    cd.step_end = (std::uint32_t)steps->size();
    cols->push_back(cd);
  }
}

template <typename T>
T* upload(const std::vector<T>& v) {
  T* d = nullptr;
  const std::size_t bytes = std::max<std::size_t>(v.size(), 1) * sizeof(T);
  QFX_CUDA(cudaMalloc(&d, bytes));
  if (!v.empty()) QFX_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return d;
}

}  // namespace

namespace {

bool overlaps(std::size_t a0, std::size_t a1, std::size_t b0, std::size_t b1) { return a0 < b1 && b0 < a1; }

// Whether the output of permute i, the A operand of product j, is read by no
// other op before it is overwritten or the program ends.
bool only_read_by(const std::vector<DevOp>& ops, std::size_t i, std::size_t j) {
  const std::size_t c0 = ops[i].c, c1 = c0 + (std::size_t(1) << ops[i].nbits);
  for (std::size_t q = i + 1; q < ops.size(); ++q) {
    const DevOp& op = ops[q];
    std::size_t w0, w1;
    if (op.kind == DevOp::PERMUTE) {
      const std::size_t sz = std::size_t(1) << op.nbits;
      if (overlaps(op.a, op.a + sz, c0, c1)) return false;
      w0 = op.c;
      w1 = op.c + sz;
    } else {
      if (q != j && overlaps(op.a, op.a + op.m * op.k, c0, c1)) return false;
      if (overlaps(op.b, op.b + op.k * op.n, c0, c1)) return false;
      w0 = op.c;
      w1 = op.c + op.m * op.n;
    }
    if (w0 <= c0 && c1 <= w1) return true;  // overwritten whole
  }
  return true;
}

}  // namespace

void Engine::plan_fusion(Plan& p) {
  const auto& ops = p.prog.ops;
  p.fused.assign(ops.size(), -1);
  p.fuse_version = options_version_;
  if (precision_ != FP16X3 || !fuse_splits_) return;
  for (std::size_t i = 0; i < ops.size(); ++i) {
    if (ops[i].kind != DevOp::PERMUTE) continue;
    // The product that reads it as A: the next op, or the one after a
    // permute of its B operand.
    for (std::size_t j = i + 1; j < ops.size() && j <= i + 2; ++j) {
      const DevOp& g = ops[j];
      if (g.kind == DevOp::PERMUTE) continue;
      if (!g.b_nk || g.a != ops[i].c || g.m * g.k != (std::size_t(1) << ops[i].nbits)) break;
      const TcConfig cfg = tc_config(g.m, g.n, g.k);
      if (g.k < 32 || (g.k & (g.k - 1)) != 0 || cfg.chunk > 2) break;
      if (only_read_by(ops, i, j)) {
        p.fused[i] = (int)j;
        p.fused[j] = (int)j;
      }
      break;
    }
  }
}

std::size_t Engine::run_program(Plan& p, int batch, float2* arena, float* tc_ws) {
  const Program& prog = p.prog;
  std::size_t launches = 0;
  const std::uint64_t stride = prog.arena_elems;
  float2* scratch = skinny_scratch();
  int* err = error_flag();
  if (profile_) {
    while (prof_events_.size() < prog.ops.size() + 1) {
      cudaEvent_t e;
      QFX_CUDA(cudaEventCreate(&e));
      prof_events_.push_back(e);
    }
  }
  if (p.fuse_version != options_version_ || p.fused.size() != prog.ops.size()) plan_fusion(p);
  for (std::size_t i = 0; i < prog.ops.size(); ++i) {
    const DevOp& op = prog.ops[i];
    if (profile_) QFX_CUDA(cudaEventRecord(prof_events_[i], stream_));
    if (op.kind == DevOp::PERMUTE) {
      if (p.fused[i] >= 0) {
        // Straight into the A planes of the product that follows.
        const DevOp& g = prog.ops[p.fused[i]];
        const Fp16Workspace w = fp16_workspace(tc_ws, g.m, g.n, g.k, batch);
        int kl = 0;
        while ((std::size_t(1) << kl) < g.k) ++kl;
        launch_permute_fp16_planes(p.perm[i], arena + op.a, stride, w.a_planes, w.a_block_exps, g.m, kl, batch,
                                   stream_);
      } else {
        launch_permute(p.perm[i], arena + op.a, arena + op.c, stride, batch, stream_);
      }
      launches += 1;
    } else if (op.b_nk) {
      const bool a_planes = p.fused[i] == (int)i;
      if (a_planes)
        launch_cgemm_fp16x3(arena + op.a, arena + op.b, arena + op.c, op.m, op.n, op.k, stride, stride, batch,
                            tc_ws, error_flag(), tc_config(op.m, op.n, op.k), stream_, true);
      else
        launch_split_product(arena + op.a, arena + op.b, arena + op.c, op.m, op.n, op.k, stride, stride, batch,
                             tc_ws);
      launches += a_planes ? 2 : 3;  // plane splits and the product
    } else {
      launch_cgemm_fp32(arena + op.a, arena + op.b, arena + op.c, op.m, op.n, op.k, stride, batch,
                        stream_, scratch);
      launches += (vm_splits(op.m, op.n, op.k, batch) || skinny_splits(op.m, op.n, op.k, batch)) ? 2 : 1;
    }
  }
  if (profile_) QFX_CUDA(cudaEventRecord(prof_events_[prog.ops.size()], stream_));
  return launches;
}

std::size_t Engine::run_program64(Plan& p, int batch, double2* arena) {
  const Program& prog = p.prog;
  std::size_t launches = 0;
  const std::uint64_t stride = prog.arena_elems;
  double2* scratch = reinterpret_cast<double2*>(skinny_scratch());
  const bool ff = precision_ == FP64_FF;
  if (profile_) {
    while (prof_events_.size() < prog.ops.size() + 1) {
      cudaEvent_t e;
      QFX_CUDA(cudaEventCreate(&e));
      prof_events_.push_back(e);
    }
  }
  for (std::size_t i = 0; i < prog.ops.size(); ++i) {
    const DevOp& op = prog.ops[i];
    if (profile_) QFX_CUDA(cudaEventRecord(prof_events_[i], stream_));
    if (op.kind == DevOp::PERMUTE) {
      launch_permute64(p.perm[i], arena + op.a, arena + op.c, stride, batch, stream_);
      launches += 1;
    } else {
      launch_zgemm(arena + op.a, arena + op.b, arena + op.c, op.m, op.n, op.k, stride, batch, stream_, scratch, ff);
      launches += zskinny_splits(op.m, op.n, op.k, batch) ? 2 : 1;
    }
  }
  if (profile_) QFX_CUDA(cudaEventRecord(prof_events_[prog.ops.size()], stream_));
  return launches;
}

std::vector<OpRecord> Engine::last_ops() const {
  std::vector<OpRecord> out;
  if (!plan_ || !plan_->built) return out;
  const Program& prog = plan_->prog;
  for (std::size_t i = 0; i < prog.ops.size(); ++i) {
    const DevOp& op = prog.ops[i];
    OpRecord r{};
    const double esize = is_complex128(plan_->precision) ? 16.0 : 8.0;
    if (op.kind == DevOp::PERMUTE) {
      r.kind = 0;
      r.m = double(std::size_t(1) << op.nbits);
      r.n = r.k = 1;
      r.bytes = 2 * esize * r.m;
    } else {
      const int nb = (int)std::max<std::size_t>(stats_.batch, 1);
      const bool split = is_complex128(plan_->precision)
                             ? zskinny_splits(op.m, op.n, op.k, nb) != 0
                             : (vm_splits(op.m, op.n, op.k, nb) || skinny_splits(op.m, op.n, op.k, nb));
      r.kind = op.b_nk ? 2 : (split ? 3 : 1);
      r.m = double(op.m);
      r.n = double(op.n);
      r.k = double(op.k);
      r.flop = 8.0 * r.m * r.n * r.k;
      r.bytes = esize * (r.m * r.k + r.k * r.n + r.m * r.n);
    }
    r.batch = double(std::max<std::size_t>(stats_.batch, 1));
    r.ms = i < op_ms_.size() ? op_ms_[i] : -1.0;
    out.push_back(r);
  }
  return out;
}

float2* Engine::skinny_scratch() {
  return (float2*)reserve(kSkinnyScratchElems * sizeof(float2), 3);
}

std::vector<EvalResult> Engine::evaluate(const std::string& circuit, const std::string& ordering,
                                         const std::string& grid, const std::string& initial_in,
                                         const std::vector<std::string>& finals,
                                         double memory_limit) {
  if (device_ >= 0) QFX_CUDA(cudaSetDevice(device_));
  if (finals.empty()) throw QFX_ERR("At least one final state is required.");
  Plan& p = *get_plan(circuit, ordering, grid);
  const long n_active = p.grid.I * p.grid.J - (long)p.grid.qubits_off.size();
  std::string initial = initial_in.empty() ? std::string((std::size_t)std::max(0L, n_active), '0')
                                           : initial_in;
  std::vector<EvalResult> results(finals.size());
  std::vector<Coord> final_qubits;
  for (std::size_t f = 0; f < finals.size(); ++f) {
    std::vector<Coord> fq;
    std::vector<std::string> states;
    std::string base;
    try {
      base = get_output_states(p.grid, p.ops, initial, finals[f], &fq, &states);
    } catch (const std::string& e) {
      throw QFX_WRAP("get_output_states", e);
    }
    results[f].initial_state = initial;
    results[f].final_state = base;
    results[f].states = std::move(states);
    if (f == 0) final_qubits = fq;
  }
  if (!p.built) {
    p.net = build_network(p.circuit, p.grid, initial, results[0].final_state, final_qubits, p.ops);
    std::function<bool(std::size_t, std::size_t, std::size_t)> b_kmajor;
    if (precision_ != FP32 && !is_complex128(precision_)) b_kmajor = tc_eligible;
    try {
      p.prog = plan_contraction(p.net, p.ops, results[0].states.size(), INFINITY, b_kmajor, open_terminals_);
    } catch (const std::string& e) {
      throw QFX_WRAP("ContractGrid", e);
    }
    p.precision = precision_;
    p.tc_ws_elems = 0;
    for (const auto& op : p.prog.ops)
      if (op.kind == DevOp::GEMM && op.b_nk)
        p.tc_ws_elems = std::max(p.tc_ws_elems, tc_workspace_elems(op.m, op.n, op.k));
    p.perm.resize(p.prog.ops.size());
    for (std::size_t i = 0; i < p.prog.ops.size(); ++i)
      if (p.prog.ops[i].kind == DevOp::PERMUTE)
        make_perm_plan(p.prog.ops[i].nbits, p.prog.ops[i].perm, &p.perm[i]);
    std::vector<ColumnDesc> cols;
    std::vector<StepDesc> steps;
    std::vector<float2> mats, mats_lo;
    std::vector<double2> mats64;
    // The plain FP32 path keeps the reference's float gate constants; the
    // split-precision path evaluates the columns from double constants (in
    // float-float), the complex128 path in FP64.
    const bool wide = is_complex128(precision_);
    const bool exact_gates = exact_gates_ < 0 ? precision_ != FP32 : exact_gates_ != 0;
    build_flatten_tables(p.net, p.prog, exact_gates, &cols, &steps, &mats, &mats_lo, wide ? &mats64 : nullptr,
                         &p.max_size_log2);
    std::vector<std::uint32_t> ptr(p.prog.n_amplitudes + 1, 0), leaves(p.prog.n_leaves);
    for (std::size_t l = 0; l < p.prog.n_leaves; ++l) ++ptr[p.prog.leaf_amp[l] + 1];
    for (std::size_t a = 0; a < p.prog.n_amplitudes; ++a) ptr[a + 1] += ptr[a];
    std::vector<std::uint32_t> fill(ptr.begin(), ptr.end() - 1);
    for (std::size_t l = 0; l < p.prog.n_leaves; ++l) leaves[fill[p.prog.leaf_amp[l]]++] = (std::uint32_t)l;
    if (device_ >= 0) {
      p.d_cols = upload(cols);
      p.d_steps = upload(steps);
      if (wide) {
        p.d_mats64 = upload(mats64);
      } else {
        p.d_mats = upload(mats);
        if (exact_gates) p.d_mats_lo = upload(mats_lo);
      }
      p.d_ptr = upload(ptr);
      p.d_leaves = upload(leaves);
    }
    p.built = true;
  } else {
    if ((long)initial.size() != n_active)
      throw QFX_ERR("Size of initial_conf: ", initial.size(),
                    ", must be equal to the number of qubits: ", n_active, ".");
  }
  for (const auto& r : results)
    if (r.final_state.size() != initial.size())
      throw QFX_ERR("Size of final_conf: ", r.final_state.size(),
                    ", must be equal to size of initial_conf: ", initial.size(), ".");
  {
    // The reference's memory-limit check (src/contraction_utils.cpp:147-155).
    const double need = p.prog.reference_bytes;
    if (need > memory_limit)
      throw QFX_WRAP("ContractGrid",
                     QFX_WRAP("Initialize", cat("Required space (", readable_memory_string(need),
                                                ") exceeds memory limit (",
                                                readable_memory_string(memory_limit),
                                                "). Cancelling simulation.")));
  }

  const Program& prog = p.prog;
  const std::size_t n_cols = p.net.columns.size();
  const std::size_t n_amps = prog.n_amplitudes;
  const bool wide = is_complex128(p.precision);
  const std::size_t arena_bytes = prog.arena_elems * (wide ? sizeof(double2) : sizeof(float2));
  const int total = (int)finals.size();

  stats_ = RunStats{};
  stats_.gemm_flop = prog.gemm_flop;
  stats_.permute_bytes = wide ? 2 * prog.permute_bytes : prog.permute_bytes;
  stats_.arena_bytes = arena_bytes;
  stats_.n_ops = prog.ops.size();
  stats_.n_leaves = prog.n_leaves;
  stats_.reference_bytes = prog.reference_bytes;
  if (device_ < 0) {  // planning-only context: amplitudes are not computed
    for (auto& r : results) r.amplitudes.assign(n_amps, {NAN, NAN});
    return results;
  }

  // How many final states fit on the device at once.
  std::size_t free_b = 0, total_b = 0;
  QFX_CUDA(cudaMemGetInfo(&free_b, &total_b));
  std::size_t have = 0;
  for (int slot : {0, 4})
    if ((int)bufs_.size() > slot) have += bufs_[slot].bytes;
  const std::size_t usable = free_b + have > (std::size_t(2) << 30) ? free_b + have - (std::size_t(2) << 30) : 0;
  const std::size_t per_entry = arena_bytes + p.tc_ws_elems * sizeof(float);
  int chunk = (int)std::max<std::size_t>(1, std::min<std::size_t>((std::size_t)total, usable / std::max<std::size_t>(per_entry, 1)));
  chunk = std::min(chunk, 65535);
  if (max_batch_ > 0) chunk = std::min(chunk, max_batch_);

  float2* arena = (float2*)reserve(arena_bytes * (std::size_t)chunk, 0);
  float* tc_ws = p.tc_ws_elems ? tc_workspace(p.tc_ws_elems * (std::size_t)chunk) : nullptr;
  skinny_scratch();
  QFX_CUDA(cudaMemsetAsync(error_flag(), 0, sizeof(int), stream_));
  double2* d_amps = (double2*)reserve(std::max<std::size_t>(n_amps, 1) * sizeof(double2) * (std::size_t)chunk, 1);
  std::uint8_t* d_bits = (std::uint8_t*)reserve(std::max<std::size_t>(n_cols, 1) * 2 * (std::size_t)chunk, 2);

  std::vector<std::uint8_t> init_bits(n_cols), bits;
  for (std::size_t c = 0; c < n_cols; ++c) {
    // Active qubits are numbered in row-major order, skipping off qubits.
    init_bits[c] = initial[c] == '0' ? 0 : 1;
  }
  std::vector<double2> h_amps(std::max<std::size_t>(n_amps, 1) * (std::size_t)chunk);
  double ms_total = 0;
  std::size_t launches = 0;
  for (int f0 = 0; f0 < total; f0 += chunk) {
    const int nb = std::min(chunk, total - f0);
    bits.assign(n_cols * 2 * (std::size_t)nb, 0);
    for (int b = 0; b < nb; ++b) {
      const std::string& fs = results[f0 + b].final_state;
      for (std::size_t c = 0; c < n_cols; ++c) {
        bits[(std::size_t)b * n_cols + c] = init_bits[c];
        bits[(std::size_t)(nb + b) * n_cols + c] = fs[c] == '0' ? 0 : 1;
      }
    }
    QFX_CUDA(cudaMemcpyAsync(d_bits, bits.data(), bits.size(), cudaMemcpyHostToDevice, stream_));
    QFX_CUDA(cudaMemsetAsync(d_amps, 0, std::max<std::size_t>(n_amps, 1) * sizeof(double2) * nb, stream_));
    QFX_CUDA(cudaEventRecord(ev0_, stream_));
    auto enqueue = [&]() -> std::size_t {
      if (wide) {
        double2* arena64 = reinterpret_cast<double2*>(arena);
        launch_flatten64(p.d_cols, (int)n_cols, p.max_size_log2, p.d_steps, p.d_mats64, d_bits,
                         d_bits + n_cols * (std::size_t)nb, arena64, prog.arena_elems, nb, stream_);
        const std::size_t l = run_program64(p, nb, arena64) + 2;  // + flatten and sums
        launch_reduce_amplitudes64(arena64 + prog.results_offset, prog.arena_elems, p.d_ptr, p.d_leaves,
                                   (int)n_amps, d_amps, nb, stream_);
        return l;
      }
      launch_flatten(p.d_cols, (int)n_cols, p.max_size_log2, p.d_steps, p.d_mats, p.d_mats_lo, d_bits,
                     d_bits + n_cols * (std::size_t)nb, arena, prog.arena_elems, nb, stream_);
      const std::size_t l = run_program(p, nb, arena, tc_ws) + 2;  // + flatten and sums
      launch_reduce_amplitudes(arena + prog.results_offset, prog.arena_elems, p.d_ptr, p.d_leaves,
                               (int)n_amps, d_amps, nb, stream_);
      return l;
    };
    // The whole pass (flatten, program, sums) is one CUDA graph once the
    // same batch size and buffers repeat: the first pass runs eagerly, the
    // second is captured, later ones replay the graph.
    const GraphKey gk{nb, arena, tc_ws, d_bits, d_amps, options_version_, precision_};
    if (!profile_ && p.graph && p.graph_key == gk) {
      QFX_CUDA(cudaGraphLaunch(p.graph, stream_));
      launches += p.graph_launches;
    } else if (!profile_ && graphs_ && p.seen_key == gk) {
      if (p.graph) cudaGraphExecDestroy(p.graph);
      p.graph = nullptr;
      cudaGraph_t g = nullptr;
      QFX_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
      std::size_t l = 0;
      try {
        l = enqueue();
      } catch (...) {
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      QFX_CUDA(cudaStreamEndCapture(stream_, &g));
      const cudaError_t ie = cudaGraphInstantiate(&p.graph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) throw cuda_error_string(ie, "cudaGraphInstantiate");
      p.graph_key = gk;
      p.graph_launches = l;
      QFX_CUDA(cudaGraphLaunch(p.graph, stream_));
      launches += l;
    } else {
      launches += enqueue();
      p.seen_key = gk;
    }
    QFX_CUDA(cudaEventRecord(ev1_, stream_));
    QFX_CUDA(cudaMemcpyAsync(h_amps.data(), d_amps, n_amps * sizeof(double2) * nb,
                             cudaMemcpyDeviceToHost, stream_));
    QFX_CUDA(cudaStreamSynchronize(stream_));
    float ms = 0;
    QFX_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
    ms_total += ms;
    if (profile_) {
      op_ms_.assign(prog.ops.size(), 0.0);
      for (std::size_t i = 0; i < prog.ops.size(); ++i) {
        float t = 0;
        QFX_CUDA(cudaEventElapsedTime(&t, prof_events_[i], prof_events_[i + 1]));
        op_ms_[i] = t;
      }
    }
    for (int b = 0; b < nb; ++b) {
      auto& r = results[f0 + b];
      r.amplitudes.resize(n_amps);
      for (std::size_t a = 0; a < n_amps; ++a) {
        const double2 v = h_amps[(std::size_t)b * n_amps + a];
        r.amplitudes[a] = {v.x, v.y};
      }
    }
  }
  if (p.tc_ws_elems) check_error_flag();
  stats_.device_ms = ms_total;
  stats_.launches = launches;
  stats_.batch = (std::size_t)chunk;
  return results;
}

}  // namespace qfx

// The contraction engine: one CUDA device, one stream, a planned HBM arena.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <map>
#include <tuple>
#include <memory>
#include <string>
#include <vector>

#include "kernels.h"
#include "tc_gemm.h"
#include "planner.h"
#include "qfx.h"

namespace qfx {

// FP64 and FP64_FF run the contraction in complex128 (the GPU oracle):
// FP64 with FP64 FMAs throughout, FP64_FF with float-float tiled products.
enum Precision : int { FP32 = 0, TF32X3 = 1, BF16X3 = 2, FP16X3 = 3, FP64 = 4, FP64_FF = 5 };
inline bool is_complex128(int precision) { return precision == FP64 || precision == FP64_FF; }

struct EvalResult {
  std::string initial_state;  // as mutated by EvaluateCircuit
  std::string final_state;
  std::vector<std::string> states;
  std::vector<std::complex<double>> amplitudes;
};

struct RunStats {
  double device_ms = 0;       // flatten + program + sums, CUDA events
  double gemm_flop = 0;       // per final state
  double permute_bytes = 0;   // per final state
  std::size_t arena_bytes = 0;  // per final state
  std::size_t n_ops = 0;
  std::size_t n_leaves = 0;
  std::size_t batch = 0;
  std::size_t launches = 0;   // kernel launches of the last evaluation
  double reference_bytes = 0;
};

// One device op of the last plan with its measured time (profiling on).
struct OpRecord {
  int kind;        // 0 permute, 1 CUDA-core product, 2 tensor-core product, 3 split-k skinny product
  double m, n, k;  // product shape (permute: m = elements)
  double flop;     // 8 m n k
  double bytes;    // operand + result bytes (permute: read + write)
  double batch;    // final states per device pass
  double ms;       // CUDA-event time of the op, -1 when not profiled
};

class Engine {
 public:
  Engine(int device, int precision);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  void set_precision(int p);
  int precision() const { return precision_; }
  void set_stream(cudaStream_t s);
  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }

  // EvaluateCircuit for one initial state and several final states (each
  // one is a separate contraction of the same network; all of them run as
  // one batch). Throws std::string on the reference's errors.
  std::vector<EvalResult> evaluate(const std::string& circuit, const std::string& ordering,
                                   const std::string& grid, const std::string& initial,
                                   const std::vector<std::string>& finals, double memory_limit);

  const RunStats& last_stats() const { return stats_; }
  // Distinct GEMM shapes of the last plan (m, n, k, count).
  const std::vector<GemmShape>& last_shapes() const;
  // The last planned program (null before the first evaluation).
  const Program* last_program() const;
  // Per-op timing: with profiling on, every device op is bracketed by CUDA
  // events (graph replay is off) and last_ops() reports each op's time.
  void set_profiling(bool on) { profile_ = on; }
  // Tuning options: "tc_chunk", "tc_pair", "graphs", "max_batch" (see the
  // C ABI). Unknown names throw.
  void set_option(const std::string& name, double value);
  double get_option(const std::string& name) const;
  // Tensor-core kernel of products of one shape (0 single CTA, 1 CTA pair,
  // -1 removes the override).
  void set_tc_variant(std::size_t m, std::size_t n, std::size_t k, int variant);
  std::vector<OpRecord> last_ops() const;

  // Device buffers owned by the engine, reused across calls.
  void* reserve(std::size_t bytes, int slot);
  // Partial-sum buffer of the split-k skinny products (kSkinnyScratchElems).
  float2* skinny_scratch();
  // Device int set by tensor-core kernels whose pipeline waits expired.
  int* error_flag();
  // Throws (and clears the flag) when a kernel reported an expired wait.
  void check_error_flag();
  // Whether the error-flag buffer exists (a tensor-core kernel may have run).
  bool has_error_flag() const { return (int)bufs_.size() > 5 && bufs_[5].ptr != nullptr; }
  // Split planes of the tensor-core products.
  float* tc_workspace(std::size_t elems);
  // C[m,n] = A[m,k] * B[k,n] (row-major complex64) in the context's
  // precision; `batch` products at `stride` elements.
  void multiply(const float2* A, const float2* B, float2* C, std::size_t m, std::size_t n,
                std::size_t k, std::uint64_t stride, int batch);

 private:
  struct Plan;
  Plan* get_plan(const std::string& circuit, const std::string& ordering, const std::string& grid);
  std::size_t run_program(Plan& p, int batch, float2* arena, float* tc_ws);
  // The same program in complex128 (FP64 and FP64_FF).
  std::size_t run_program64(Plan& p, int batch, double2* arena);
  // Marks permute/product pairs whose A operand goes straight into planes.
  void plan_fusion(Plan& p);

  int device_;
  int precision_;
  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  bool graphs_ = true;  // capture repeated device passes (QFLEX_GB300_GRAPHS=0 disables)
  bool profile_ = false;
  TcConfig tc_cfg_;
  std::map<std::tuple<std::size_t, std::size_t, std::size_t>, int> tc_variant_;
  int max_batch_ = 0;            // output strings per device pass (0: as many as fit)
  bool open_terminals_ = true;   // terminal cuts as open indices where the planner can
  bool fuse_splits_ = true;      // 3xFP16: permutes write the next product's A planes
  unsigned long long wait_ns_ = 0;  // tensor-core pipeline wait limit (0: the kernels' 2 s)
  int exact_gates_ = -1;  // gate tensors from double constants: -1 all but FP32, 0 never, 1 always
  bool debias_ = true;    // tensor-core products compensate the truncation bias
  unsigned options_version_ = 0;  // part of the graph key: options change launches
  TcConfig tc_config(std::size_t m, std::size_t n, std::size_t k) const;
  // C = A * Bt^T on the tensor cores in the context's split precision.
  void launch_split_product(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                            std::size_t k, std::uint64_t ac_stride, std::uint64_t bt_stride, int batch, float* ws);
  std::vector<cudaEvent_t> prof_events_;
  std::vector<double> op_ms_;
  std::unique_ptr<Plan> plan_;
  struct DevBuf {
    void* ptr = nullptr;
    std::size_t bytes = 0;
  };
  std::vector<DevBuf> bufs_;
  RunStats stats_;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
};

std::string cuda_error_string(cudaError_t e, const char* what);

}  // namespace qfx

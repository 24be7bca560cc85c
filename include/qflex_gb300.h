/*
 * qflex_gb300 — C ABI of the GB300 engine for qFlex grid tensor-network
 * contraction (random quantum circuit amplitudes).
 *
 * Plain pointers and sizes only; no exception crosses this boundary. Every
 * function returns QFLEX_GB300_OK or an error code, and the message of the
 * last failure is available from qflex_gb300_last_error(). Reference errors
 * (bad circuit, grid or ordering text, memory limit, ...) carry the same
 * message text as the reference's thrown std::string.
 *
 * One context = one CUDA device + one stream; a context must be used from
 * one thread at a time (the reference itself is not thread-safe:
 * src/tensor.cpp:83, src/global.h:9-15).
 *
 * Citations are paths inside the ngnrsaa/qflex project.
 */
#ifndef QFLEX_GB300_H
#define QFLEX_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QFLEX_GB300_OK 0
#define QFLEX_GB300_ERR_INPUT 1 /* the reference would throw std::string */
#define QFLEX_GB300_ERR_CUDA 2  /* CUDA runtime failure */
#define QFLEX_GB300_ERR_ARG 3   /* invalid argument to this API */

/* Arithmetic of the complex64 contractions. */
#define QFLEX_GB300_FP32 0   /* FP32 CUDA cores (matches complex<float>) */
#define QFLEX_GB300_TF32X3 1 /* split 3xTF32 on tcgen05 tensor cores */
#define QFLEX_GB300_BF16X3 2 /* split BF16x3 (six products per real product) on tcgen05 tensor cores */
#define QFLEX_GB300_FP16X3 3 /* split 3xFP16 (rows scaled by powers of two) on tcgen05 tensor cores */
/* The FP64 GPU oracle: the same contraction in complex128 (double gate
 * constants, complex128 tensors in HBM, FP64 amplitude sums). The reference
 * has no FP64 mode (its s_type is std::complex<float>, src/tensor.h:29). */
#define QFLEX_GB300_FP64 4    /* every product with FP64 FMAs */
#define QFLEX_GB300_FP64_FF 5 /* tiled products in float-float (~44 bits) on the FP32 pipes, rest FP64 */

typedef struct qflex_gb300_context qflex_gb300_context;

typedef struct {
  double device_ms;       /* device time of the last evaluation */
  double gemm_flop;       /* 8*m*n*k summed over products, per final state */
  double permute_bytes;   /* 16*size summed over permutes, per final state */
  double arena_bytes;     /* HBM arena of one final state */
  double reference_bytes; /* the reference's planned scratch (memory check) */
  size_t n_ops;           /* device ops of the program */
  size_t n_leaves;        /* contraction leaves (cut slices x terminal values) */
  size_t batch;           /* final states evaluated per device pass */
  size_t launches;        /* kernel launches of the last evaluation */
} qflex_gb300_stats;

/* Creates a context on CUDA device `device`. No reference counterpart (the
 * reference allocates per call inside ContractGrid,
 * src/contraction_utils.cpp:612-639). device = -1 creates a planning-only
 * context: evaluations parse, validate and plan (errors, output states,
 * statistics, product shapes) without touching a GPU, and amplitudes are
 * NaN. */
int qflex_gb300_create(int device, int precision, qflex_gb300_context** out);
void qflex_gb300_destroy(qflex_gb300_context* ctx);
const char* qflex_gb300_last_error(const qflex_gb300_context* ctx);
int qflex_gb300_set_precision(qflex_gb300_context* ctx, int precision);
/* Runs all work of this context on `stream` (a cudaStream_t); NULL restores
 * the context's own stream. */
int qflex_gb300_set_stream(qflex_gb300_context* ctx, void* stream);

/* Replaces qflex::EvaluateCircuit(QflexInput*)
 * (src/evaluate_circuit.h:81-82, src/evaluate_circuit.cpp:106-253).
 * `circuit`, `ordering`, `grid` are the texts of the three input files
 * (formats of src/circuit.cpp:30-206, src/ordering.cpp:10-45,
 * src/grid.cpp:11-45; docs/input_formats.md). `initial_state` and
 * `final_state` may be empty, as in QflexInput (src/input.h:11-17).
 * `memory_limit` in bytes plays the role of global::memory_limit
 * (src/global.h:12); <= 0 means the reference default of 1 GiB.
 * Results are kept in the context (see the accessors below). */
int qflex_gb300_evaluate(qflex_gb300_context* ctx, const char* circuit, const char* ordering,
                         const char* grid, const char* initial_state, const char* final_state,
                         double memory_limit);

/* The batched form: one contraction per final state, all of them run as one
 * device batch. Each final state gives the amplitudes EvaluateCircuit would
 * return for it; results are concatenated in input order. The reference has
 * no batched call; its pybind layer rejects several final states
 * (src/pybind_main.cpp:111-113), and callers loop instead
 * (qflexcirq/interface/qflex_simulator.py:44-53). */
int qflex_gb300_evaluate_many(qflex_gb300_context* ctx, const char* circuit, const char* ordering,
                              const char* grid, const char* initial_state,
                              const char* const* final_states, size_t n_final_states,
                              double memory_limit);

/* Results of the last evaluation: the (state, amplitude) pairs of
 * src/evaluate_circuit.cpp:245-247, and the mutated initial/final states of
 * QflexInput (src/evaluate_circuit.cpp:130-145). */
size_t qflex_gb300_result_count(const qflex_gb300_context* ctx);
const char* qflex_gb300_result_state(const qflex_gb300_context* ctx, size_t i);
int qflex_gb300_result_amplitude(const qflex_gb300_context* ctx, size_t i, double* re, double* im);
const char* qflex_gb300_result_initial_state(const qflex_gb300_context* ctx);
/* Mutated final state of final state number `which` of the last call. */
const char* qflex_gb300_result_final_state(const qflex_gb300_context* ctx, size_t which);
int qflex_gb300_last_stats(const qflex_gb300_context* ctx, qflex_gb300_stats* out);
/* Distinct product shapes of the last plan: writes up to `cap` rows of
 * (m, n, k, count) into `out` and returns the number of distinct shapes. */
size_t qflex_gb300_last_shapes(const qflex_gb300_context* ctx, size_t* out, size_t cap);
/* Every product of the last plan in execution order: up to `cap` rows of
 * (m, n, k). These are the (m, n, k) the reference passes to cblas_cgemm,
 * cgemv and cdotu_sub inside ContractGrid (src/tensor.cpp:973-1041), in the
 * same order. Returns the number of products. */
size_t qflex_gb300_last_gemms(const qflex_gb300_context* ctx, size_t* out, size_t cap);

/* Per-op timing, the engine's counterpart of the reference's verbose
 * per-multiply timings ("[R] reordering", "[M] multiplying",
 * src/tensor.cpp:1059-1193). With profiling on, every device op of an
 * evaluation is bracketed by CUDA events (captured graphs are not used).
 * qflex_gb300_last_ops writes up to `cap` rows of 8 doubles per op of the
 * last plan -- kind (0 permute, 1 CUDA-core product, 2 tensor-core product,
 * 3 split-k skinny product), m, n, k (permute: m = elements), flop, bytes,
 * batch, milliseconds (-1 if not profiled) -- and returns the op count. */
int qflex_gb300_set_profiling(qflex_gb300_context* ctx, int on);
size_t qflex_gb300_last_ops(const qflex_gb300_context* ctx, double* out, size_t cap);

/* Tuning options of a context; no reference counterpart (the reference has
 * no device kernels to tune). Names and values:
 *   "tc_chunk"   k-steps per TMEM accumulation chunk of the split
 *                tensor-core product, 1..64 (default 2, or QFLEX_TC_CHUNK;
 *                longer chunks are faster and less accurate: the tensor
 *                core's FP32 accumulation truncates, which shrinks every
 *                product by an amount that grows with the chunk)
 *   "tc_pair"    1: 3xTF32 products with m >= 256 use the CTA-pair
 *                (cta_group::2, 256 x 128 tile) kernel; 0: every product uses
 *                the single-CTA 128 x 128 tile (default 0, or QFLEX_TC_PAIR)
 *   "tc_variant" tensor-core kernel of every product without a per-shape
 *                choice (qflex_gb300_set_tc_variant): 0..4 as listed there
 *                (default 0; "tc_pair" sets 0 or the pair-for-m >= 256 rule)
 *   "graphs"     1: capture a repeated device pass in a CUDA graph and
 *                replay it (default 1, or QFLEX_GB300_GRAPHS)
 *   "max_batch"  most output strings per device pass of evaluate_many
 *                (0: as many as fit in device memory; default 0)
 *   "fuse_splits" 1 (3xFP16): a permutation whose output is the next
 *                product's A operand and read by nothing else writes the FP16
 *                planes (scaled per 32 values of a row) directly instead of
 *                complex64, and the product skips splitting A (default 1,
 *                or QFLEX_GB300_FUSE)
 *   "tc_debias"  1: the split tensor-core products multiply their outputs
 *                by 1 + beta, the mean fraction the tensor core's truncating
 *                accumulation loses (measured on GB300 per split kind for
 *                chunks of 1 and 2 k-steps on Gaussian operands; other
 *                chunk lengths are not compensated); 0: no compensation
 *                (default 1)
 *   "exact_gates" -1: the plain FP32 path builds its gate tensors from the
 *                reference's float gate constants, every other mode from double
 *                constants (default); 1: every mode from double constants; 0:
 *                every complex64 mode from float constants
 *   "tc_wait_ns" limit in ns of every pipeline wait of the tensor-core
 *                products (0: 2 s, the default). A wait that runs out stops its
 *                thread block, which drains the copies and MMAs it started,
 *                frees its tensor memory and returns; the call (or the next
 *                qflex_gb300_synchronize after qflex_gb300_multiply) returns
 *                QFLEX_GB300_ERR_CUDA, "tensor-core pipeline wait expired", and
 *                the context stays usable. For tests of that path.
 *   "open_terminals" 1: terminal cuts that take all their values, with no
 *                two-qubit cut after them, stay open indices -- the ops after
 *                them run once on tensors carrying the open indices instead
 *                of once per terminal value (same amplitudes); 0: the
 *                reference's projection per value (default 1)
 * Unknown names and out-of-range values return QFLEX_GB300_ERR_ARG. */
int qflex_gb300_set_option(qflex_gb300_context* ctx, const char* name, double value);
int qflex_gb300_get_option(const qflex_gb300_context* ctx, const char* name, double* value);
/* Tensor-core kernel for products of shape (m, n, k), e.g. chosen by an
 * autotuner: 0 single CTA, 1 CTA pair (needs m >= 64), 2 single CTA with a
 * deeper operand pipeline (3xFP16), 3 single CTA with 16 epilogue warps
 * (3xFP16; outputs that cannot take bulk tensor stores use 0), 4 single CTA
 * with 64-column tiles and four TMEM chunk buffers (3xFP16); the other
 * precisions take 0. -1 removes the override. Overrides "tc_pair" for that
 * shape. */
int qflex_gb300_set_tc_variant(qflex_gb300_context* ctx, size_t m, size_t n, size_t k, int variant);

/* ---- tensor-level operations on device memory (complex64, interleaved) ----
 * Pointers are CUDA device pointers; work is queued on the context's stream.
 * They need a complex64 precision mode (not QFLEX_GB300_FP64 / _FP64_FF).
 */

/* Out-of-place index permutation: the data movement of Tensor::reorder
 * (src/tensor.cpp:866-911). The tensor has `rank` indices with dimensions
 * `dims` (row-major, last index fastest); `new_order[i]` is the old position
 * of the index that goes to position i. `batch` tensors at a distance of
 * `batch_stride` elements are permuted. When every dimension is a power of
 * two (the only dimensions a contraction creates) the tiled binary-digit
 * kernel runs (the reference's _fast_reorder, src/tensor.cpp:494-864);
 * otherwise a general gather kernel (its _naive_reorder,
 * src/tensor.cpp:377-492), for at most 32 indices. */
int qflex_gb300_permute(qflex_gb300_context* ctx, const void* src, void* dst, size_t rank,
                        const size_t* dims, const size_t* new_order, size_t batch,
                        size_t batch_stride);

/* Host-side check of the permutation kernels' index math: runs the chosen
 * kernel's exact schedule (same tables, same tile order, or the general
 * kernel's index decomposition) over HOST buffers of complex64. For tests
 * and diagnostics; needs no GPU and no context. No reference counterpart. */
int qflex_gb300_check_permute(size_t rank, const size_t* dims, const size_t* new_order,
                              const void* src_host, void* dst_host);

/* In-place reorder with caller-provided scratch of at least the tensor's
 * size: Tensor::reorder(new_ordering, scratch_copy) (src/tensor.h:215,
 * src/tensor.cpp:866-911). Afterwards `data` holds the permuted tensor. */
int qflex_gb300_reorder(qflex_gb300_context* ctx, void* data, void* scratch, size_t rank,
                        const size_t* dims, const size_t* new_order);

/* C[m,n] = A[m,k] * B[k,n], row-major complex64, alpha = 1, beta = 0: the
 * products multiply() hands to cblas_cgemm / cgemv / cdotu_sub
 * (src/tensor.cpp:960-1042). `batch` products at a distance of
 * `batch_stride` elements. */
int qflex_gb300_multiply(qflex_gb300_context* ctx, const void* A, const void* B, void* C, size_t m,
                         size_t n, size_t k, size_t batch, size_t batch_stride);

int qflex_gb300_synchronize(qflex_gb300_context* ctx);

/* ---- the input models, parsed ----
 * The reference's QflexCircuit / QflexGrid / QflexOrdering parse their text
 * in load() and expose the parsed members (src/circuit.h, src/grid.h,
 * src/ordering.h); these functions run the parsers EvaluateCircuit uses and
 * return the same members. Errors return QFLEX_GB300_ERR_INPUT with the
 * reference's message in `err` (`err_len` bytes, may be NULL). */
typedef struct qflex_gb300_circuit qflex_gb300_circuit;
/* QflexCircuit::load (src/circuit.cpp:30-206). Free with
 * qflex_gb300_circuit_free. */
int qflex_gb300_circuit_load(const char* text, qflex_gb300_circuit** out, char* err, size_t err_len);
void qflex_gb300_circuit_free(qflex_gb300_circuit* circuit);
/* QflexCircuit::num_active_qubits, depth and gates.size(). */
size_t qflex_gb300_circuit_num_active_qubits(const qflex_gb300_circuit* circuit);
size_t qflex_gb300_circuit_depth(const qflex_gb300_circuit* circuit);
size_t qflex_gb300_circuit_gate_count(const qflex_gb300_circuit* circuit);
/* Gate `i` (QflexGate, src/circuit.h): `name` and `raw` (the cleaned line)
 * stay owned by `circuit`; up to `qubits_cap` qubits and `params_cap`
 * parameters are written, and their full counts go to *n_qubits and
 * *n_params. */
int qflex_gb300_circuit_gate(const qflex_gb300_circuit* circuit, size_t i, const char** name, const char** raw,
                             size_t* cycle, size_t* qubits, size_t qubits_cap, size_t* n_qubits, double* params,
                             size_t params_cap, size_t* n_params);
/* QflexGrid::load (src/grid.cpp:11-45): I, J and the off qubits as
 * (row, column) pairs, up to `off_cap` pairs into `off`; *n_off gets the
 * full count. */
int qflex_gb300_grid_load(const char* text, size_t* I, size_t* J, size_t* off, size_t off_cap, size_t* n_off,
                          char* err, size_t err_len);
/* QflexOrdering::load (src/ordering.cpp:10-45): the cleaned instruction
 * lines joined by '\n' into `out` (NUL-terminated, at most `cap` bytes);
 * *needed gets the bytes required including the NUL, *n_instructions the
 * number of lines. */
int qflex_gb300_ordering_load(const char* text, char* out, size_t cap, size_t* n_instructions, size_t* needed,
                              char* err, size_t err_len);

/* ---- learned cost model kernels ----
 * A 3-layer perceptron y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 in FP32
 * that predicts an op's log time from its features; it ranks candidate
 * orderings the way the reference's auto-orderer ranks them with its
 * analytic cost (qflexcirq/ordering/order_circuit_simulation.py:87-106).
 * No counterpart in the reference's C++ core. All pointers are device
 * pointers; work is queued on `stream`. `work` holds
 * qflex_gb300_mlp_work_floats(n, hidden) floats. */
size_t qflex_gb300_mlp_param_count(int d_in, int hidden);
size_t qflex_gb300_mlp_work_floats(size_t n, int hidden);
int qflex_gb300_mlp_forward(void* stream, const float* params, const float* X, size_t n, int d_in, int hidden,
                            float* work, float* y);
/* Mean-squared error against `target` (written to *loss, device) and its
 * gradient with respect to every parameter (written to `grads`). */
int qflex_gb300_mlp_loss_grad(void* stream, const float* params, const float* X, const float* target, size_t n,
                              int d_in, int hidden, float* work, float* grads, float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8); `step` counts from 1. */
int qflex_gb300_mlp_adam(void* stream, float* params, const float* grads, float* m, float* v, size_t count,
                         int step, float lr);

/* Skinny product that allocates no device memory: C[m,n] = A[m,k] * B[k,n]
 * (row-major complex64) for at most 64 outputs (m * n <= 64, m, n <= 64),
 * i.e. the dot products and narrow matrix-vector products that multiply()
 * hands to cblas_cgemv / cblas_cdotu_sub. This one has no counterpart in
 * the reference: it exists for callers that must not allocate, because
 * cudaMalloc / cudaFree may synchronize the whole device or the caller has
 * no memory budget left to give. It takes no context; work is queued on
 * `stream` (a cudaStream_t, NULL for the legacy stream) of the current
 * device.
 *
 * The split-k partial sums go to one fixed array of 65536 complex64 slots
 * (512 KiB) compiled into the library; every GPU that loads the library
 * holds it until the process exits. The first call made with a device
 * current looks up that device's copy of the array (cudaGetSymbolAddress);
 * make that first call before any stream capture. All calls share the
 * array: calls that overlap on the GPU (other streams, other threads) race
 * and corrupt each other's results, so serialize them. Every slot a call
 * reads is written by that call first, so nothing needs clearing. Sizes
 * beyond the limits return QFLEX_GB300_ERR_ARG with a message in `err`
 * (`err_len` bytes, may be NULL). */
int qflex_gb300_multiply_skinny_noalloc(const void* A, const void* B, void* C, size_t m, size_t n,
                                        size_t k, void* stream, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* QFLEX_GB300_H */

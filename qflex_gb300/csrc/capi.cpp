// extern "C" boundary of the engine (declared in include/qflex_gb300.h).
// Converts thrown std::string / std::exception into status codes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>

#include "../../include/qflex_gb300.h"
#include "engine.h"

struct qflex_gb300_context {
  std::unique_ptr<qfx::Engine> engine;
  std::string error;
  std::string initial;
  std::vector<std::string> finals;
  std::vector<std::string> states;
  std::vector<std::complex<double>> amps;
};

namespace {

constexpr double kDefaultMemoryLimit = double(1ull << 30);

template <typename F>
int guarded(qflex_gb300_context* ctx, F&& f) {
  if (!ctx) return QFLEX_GB300_ERR_ARG;
  try {
    f();
    ctx->error.clear();
    return QFLEX_GB300_OK;
  } catch (const std::string& e) {
    ctx->error = e;
    return e.rfind("ERROR (qflex_gb300: CUDA", 0) == 0 ? QFLEX_GB300_ERR_CUDA : QFLEX_GB300_ERR_INPUT;
  } catch (const char* e) {
    ctx->error = e;
    return QFLEX_GB300_ERR_INPUT;
  } catch (const std::bad_alloc&) {
    ctx->error = "ERROR (qflex_gb300) --> host allocation failed";
    return QFLEX_GB300_ERR_ARG;
  } catch (const std::exception& e) {
    ctx->error = e.what();
    return QFLEX_GB300_ERR_INPUT;
  } catch (...) {  // nothing may cross the C ABI
    ctx->error = "ERROR (qflex_gb300) --> unknown exception";
    return QFLEX_GB300_ERR_INPUT;
  }
}

void store(qflex_gb300_context* ctx, std::vector<qfx::EvalResult>&& res) {
  ctx->states.clear();
  ctx->amps.clear();
  ctx->finals.clear();
  ctx->initial = res.empty() ? std::string() : res[0].initial_state;
  for (auto& r : res) {
    ctx->finals.push_back(r.final_state);
    for (std::size_t i = 0; i < r.states.size(); ++i) {
      ctx->states.push_back(r.states[i]);
      ctx->amps.push_back(r.amplitudes[i]);
    }
  }
}

bool all_powers_of_two(std::size_t rank, const std::size_t* dims) {
  for (std::size_t i = 0; i < rank; ++i)
    if (dims[i] == 0 || (dims[i] & (dims[i] - 1)) != 0) return false;
  return true;
}

// A permutation of any dimensions: the binary-digit plan when every
// dimension is a power of two, the general gather otherwise.
struct AnyPerm {
  bool binary = true;
  int nbits = 0;
  qfx::PermPlan plan;
  qfx::GeneralPerm general;
  std::uint64_t size() const { return binary ? (std::uint64_t(1) << nbits) : general.size; }
};

void check_perm(std::size_t rank, const std::size_t* dims, const std::size_t* order, int* nbits,
                std::uint8_t* perm);

void plan_any_perm(std::size_t rank, const std::size_t* dims, const std::size_t* order, AnyPerm* out,
                   bool* identity = nullptr) {
  if (rank > 0 && (!dims || !order)) throw QFX_ERR("dims and new_order must be non-null.");
  if (all_powers_of_two(rank, dims)) {
    std::uint8_t perm[40] = {};
    check_perm(rank, dims, order, &out->nbits, perm);
    out->binary = true;
    qfx::make_perm_plan(out->nbits, perm, &out->plan);
    if (identity) {
      *identity = true;
      for (int b = 0; b < out->nbits; ++b) *identity &= perm[b] == b;
    }
  } else {
    out->binary = false;
    qfx::make_general_perm(rank, dims, order, &out->general);
    if (identity) {
      *identity = true;
      for (std::size_t i = 0; i < rank; ++i) *identity &= order[i] == i;
    }
  }
}

void launch_any_perm(const AnyPerm& p, const float2* src, float2* dst, std::uint64_t batch_stride, int batch,
                     cudaStream_t s) {
  if (p.binary)
    qfx::launch_permute(p.plan, src, dst, batch_stride, batch, s);
  else
    qfx::launch_permute_general(p.general, src, dst, batch_stride, batch, s);
}

void check_perm(std::size_t rank, const std::size_t* dims, const std::size_t* order, int* nbits,
                std::uint8_t* perm) {
  if (rank > 0 && (!dims || !order)) throw QFX_ERR("dims and new_order must be non-null.");
  std::vector<int> lg(rank);
  int total = 0;
  std::vector<bool> seen(rank, false);
  for (std::size_t i = 0; i < rank; ++i) {
    int l = 0;
    while ((std::size_t(1) << l) < dims[i]) ++l;
    if ((std::size_t(1) << l) != dims[i]) throw QFX_ERR("Dimension ", dims[i], " is not a power of two.");
    lg[i] = l;
    total += l;
    if (order[i] >= rank || seen[order[i]])
      throw QFX_ERR("new_order must be a permutation of 0..", rank - 1, ".");
    seen[order[i]] = true;
  }
  if (total > 31) throw QFX_ERR("Tensor of 2^", total, " elements is too large.");
  std::vector<int> s_old(rank, 0), s_new(rank, 0), new_pos(rank);
  for (std::size_t i = rank; i-- > 1;) s_old[i - 1] = s_old[i] + lg[i];
  for (std::size_t p = 0; p < rank; ++p) new_pos[order[p]] = (int)p;
  for (std::size_t p = rank; p-- > 1;) s_new[p - 1] = s_new[p] + lg[order[p]];
  for (std::size_t i = 0; i < rank; ++i)
    for (int b = 0; b < lg[i]; ++b) perm[s_old[i] + b] = (std::uint8_t)(s_new[new_pos[i]] + b);
  *nbits = total;
}

}  // namespace

extern "C" {

int qflex_gb300_create(int device, int precision, qflex_gb300_context** out) {
  if (!out) return QFLEX_GB300_ERR_ARG;
  *out = nullptr;
  auto* ctx = new (std::nothrow) qflex_gb300_context();
  if (!ctx) return QFLEX_GB300_ERR_ARG;
  int rc = guarded(ctx, [&] { ctx->engine = std::make_unique<qfx::Engine>(device, precision); });
  *out = ctx;  // returned even on failure so the error text can be read
  return rc;
}

void qflex_gb300_destroy(qflex_gb300_context* ctx) { delete ctx; }

const char* qflex_gb300_last_error(const qflex_gb300_context* ctx) {
  return ctx ? ctx->error.c_str() : "null context";
}

int qflex_gb300_set_precision(qflex_gb300_context* ctx, int precision) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    ctx->engine->set_precision(precision);
  });
}

int qflex_gb300_set_stream(qflex_gb300_context* ctx, void* stream) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    if (stream) {
      ctx->engine->set_stream((cudaStream_t)stream);
    } else {
      cudaStream_t s;
      cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      if (e != cudaSuccess) throw qfx::cuda_error_string(e, "cudaStreamCreate");
      ctx->engine->set_stream(s);
    }
  });
}

int qflex_gb300_evaluate(qflex_gb300_context* ctx, const char* circuit, const char* ordering,
                         const char* grid, const char* initial_state, const char* final_state,
                         double memory_limit) {
  const char* finals[1] = {final_state ? final_state : ""};
  return qflex_gb300_evaluate_many(ctx, circuit, ordering, grid, initial_state, finals, 1,
                                   memory_limit);
}

int qflex_gb300_evaluate_many(qflex_gb300_context* ctx, const char* circuit, const char* ordering,
                              const char* grid, const char* initial_state,
                              const char* const* final_states, size_t n_final_states,
                              double memory_limit) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    if (!final_states && n_final_states) throw QFX_ERR("final_states must be non-null.");
    std::vector<std::string> finals;
    for (size_t i = 0; i < n_final_states; ++i) finals.emplace_back(final_states[i] ? final_states[i] : "");
    const double limit = memory_limit > 0 ? memory_limit : kDefaultMemoryLimit;
    store(ctx, ctx->engine->evaluate(circuit ? circuit : "", ordering ? ordering : "",
                                     grid ? grid : "", initial_state ? initial_state : "", finals,
                                     limit));
  });
}

size_t qflex_gb300_result_count(const qflex_gb300_context* ctx) { return ctx ? ctx->amps.size() : 0; }

const char* qflex_gb300_result_state(const qflex_gb300_context* ctx, size_t i) {
  return (ctx && i < ctx->states.size()) ? ctx->states[i].c_str() : nullptr;
}

int qflex_gb300_result_amplitude(const qflex_gb300_context* ctx, size_t i, double* re, double* im) {
  if (!ctx || i >= ctx->amps.size() || !re || !im) return QFLEX_GB300_ERR_ARG;
  *re = ctx->amps[i].real();
  *im = ctx->amps[i].imag();
  return QFLEX_GB300_OK;
}

const char* qflex_gb300_result_initial_state(const qflex_gb300_context* ctx) {
  return ctx ? ctx->initial.c_str() : nullptr;
}

const char* qflex_gb300_result_final_state(const qflex_gb300_context* ctx, size_t which) {
  return (ctx && which < ctx->finals.size()) ? ctx->finals[which].c_str() : nullptr;
}

int qflex_gb300_last_stats(const qflex_gb300_context* ctx, qflex_gb300_stats* out) {
  if (!ctx || !out || !ctx->engine) return QFLEX_GB300_ERR_ARG;
  const auto& s = ctx->engine->last_stats();
  out->device_ms = s.device_ms;
  out->gemm_flop = s.gemm_flop;
  out->permute_bytes = s.permute_bytes;
  out->arena_bytes = double(s.arena_bytes);
  out->reference_bytes = s.reference_bytes;
  out->n_ops = s.n_ops;
  out->n_leaves = s.n_leaves;
  out->batch = s.batch;
  out->launches = s.launches;
  return QFLEX_GB300_OK;
}

size_t qflex_gb300_last_shapes(const qflex_gb300_context* ctx, size_t* out, size_t cap) {
  if (!ctx || !ctx->engine) return 0;
  const auto& shapes = ctx->engine->last_shapes();
  for (size_t i = 0; i < shapes.size() && i < cap && out; ++i) {
    out[4 * i + 0] = shapes[i].m;
    out[4 * i + 1] = shapes[i].n;
    out[4 * i + 2] = shapes[i].k;
    out[4 * i + 3] = shapes[i].count;
  }
  return shapes.size();
}

size_t qflex_gb300_last_gemms(const qflex_gb300_context* ctx, size_t* out, size_t cap) {
  if (!ctx || !ctx->engine || !ctx->engine->last_program()) return 0;
  size_t n = 0;
  for (const auto& op : ctx->engine->last_program()->ops) {
    if (op.kind != qfx::DevOp::GEMM) continue;
    if (out && n < cap) {
      out[3 * n + 0] = op.m;
      out[3 * n + 1] = op.n;
      out[3 * n + 2] = op.k;
    }
    ++n;
  }
  return n;
}

int qflex_gb300_set_option(qflex_gb300_context* ctx, const char* name, double value) {
  if (!name) return QFLEX_GB300_ERR_ARG;
  int rc = guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    ctx->engine->set_option(name, value);
  });
  return rc == QFLEX_GB300_ERR_INPUT ? QFLEX_GB300_ERR_ARG : rc;
}

int qflex_gb300_get_option(const qflex_gb300_context* ctx, const char* name, double* value) {
  if (!ctx || !ctx->engine || !name || !value) return QFLEX_GB300_ERR_ARG;
  try {
    *value = ctx->engine->get_option(name);
  } catch (...) {
    return QFLEX_GB300_ERR_ARG;
  }
  return QFLEX_GB300_OK;
}

int qflex_gb300_set_tc_variant(qflex_gb300_context* ctx, size_t m, size_t n, size_t k, int variant) {
  int rc = guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    ctx->engine->set_tc_variant(m, n, k, variant);
  });
  return rc == QFLEX_GB300_ERR_INPUT ? QFLEX_GB300_ERR_ARG : rc;
}

int qflex_gb300_set_profiling(qflex_gb300_context* ctx, int on) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    ctx->engine->set_profiling(on != 0);
  });
}

size_t qflex_gb300_last_ops(const qflex_gb300_context* ctx, double* out, size_t cap) {
  if (!ctx || !ctx->engine) return 0;
  try {  // the op list is built on the host: nothing may cross the C ABI
    const auto ops = ctx->engine->last_ops();
    for (size_t i = 0; i < ops.size() && i < cap && out; ++i) {
      const auto& r = ops[i];
      const double row[8] = {double(r.kind), r.m, r.n, r.k, r.flop, r.bytes, r.batch, r.ms};
      std::memcpy(out + 8 * i, row, sizeof(row));
    }
    return ops.size();
  } catch (...) {
    return 0;
  }
}

int qflex_gb300_permute(qflex_gb300_context* ctx, const void* src, void* dst, size_t rank,
                        const size_t* dims, const size_t* new_order, size_t batch,
                        size_t batch_stride) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    if (!src || !dst) throw QFX_ERR("Data pointers must be non-null.");
    if (src == dst) throw QFX_ERR("src and dst must not overlap; use qflex_gb300_reorder.");
    if (batch == 0) return;
    if (batch > 65535) throw QFX_ERR("batch must be at most 65535.");
    if (qfx::is_complex128(ctx->engine->precision()))
      throw QFX_ERR("The complex64 tensor operations need a complex64 precision mode (this context is complex128).");
    AnyPerm p;
    plan_any_perm(rank, dims, new_order, &p);
    cudaSetDevice(ctx->engine->device());
    launch_any_perm(p, (const float2*)src, (float2*)dst, batch_stride, (int)batch, ctx->engine->stream());
  });
}

int qflex_gb300_check_permute(size_t rank, const size_t* dims, const size_t* new_order,
                              const void* src_host, void* dst_host) {
  try {
    if (!src_host || !dst_host) return QFLEX_GB300_ERR_ARG;
    AnyPerm p;
    plan_any_perm(rank, dims, new_order, &p);
    if (p.binary)
      qfx::permute_schedule_on_host(p.plan, (const float2*)src_host, (float2*)dst_host, p.size());
    else
      qfx::permute_general_on_host(p.general, (const float2*)src_host, (float2*)dst_host);
    return QFLEX_GB300_OK;
  } catch (...) {
    return QFLEX_GB300_ERR_ARG;
  }
}

int qflex_gb300_reorder(qflex_gb300_context* ctx, void* data, void* scratch, size_t rank,
                        const size_t* dims, const size_t* new_order) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    if (!scratch) throw QFX_ERR("Scratch copy must be non-null.");
    if (!data) throw QFX_ERR("Data must be non-null.");
    if (qfx::is_complex128(ctx->engine->precision()))
      throw QFX_ERR("The complex64 tensor operations need a complex64 precision mode (this context is complex128).");
    AnyPerm p;
    bool identity = false;
    plan_any_perm(rank, dims, new_order, &p, &identity);
    if (identity) return;
    cudaSetDevice(ctx->engine->device());
    launch_any_perm(p, (const float2*)data, (float2*)scratch, 0, 1, ctx->engine->stream());
    cudaError_t e = cudaMemcpyAsync(data, scratch, p.size() * sizeof(float2), cudaMemcpyDeviceToDevice,
                                    ctx->engine->stream());
    if (e != cudaSuccess) throw qfx::cuda_error_string(e, "cudaMemcpyAsync");
  });
}

int qflex_gb300_multiply(qflex_gb300_context* ctx, const void* A, const void* B, void* C, size_t m,
                         size_t n, size_t k, size_t batch, size_t batch_stride) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    if (!A) throw QFX_ERR("Data from Tensor A must be non-null.");
    if (!B) throw QFX_ERR("Data from Tensor B must be non-null.");
    if (!C) throw QFX_ERR("Data from Tensor C must be non-null.");
    if (A == C) throw QFX_ERR("A and C cannot be the same tensor.");
    if (B == C) throw QFX_ERR("B and C cannot be the same tensor.");
    if (batch == 0 || m == 0 || n == 0) return;
    if (batch > 65535) throw QFX_ERR("batch must be at most 65535.");
    cudaSetDevice(ctx->engine->device());
    ctx->engine->multiply((const float2*)A, (const float2*)B, (float2*)C, m, n, k, batch_stride,
                          (int)batch);
  });
}

}  // extern "C"

struct qflex_gb300_circuit {
  qfx::Circuit circuit;
};

namespace {

// Runs a parser; reference errors become QFLEX_GB300_ERR_INPUT with the
// message in `err`.
template <typename F>
int parse_guarded(char* err, std::size_t err_len, F&& f) {
  auto put = [&](const std::string& msg) {
    if (err && err_len) {
      std::strncpy(err, msg.c_str(), err_len - 1);
      err[err_len - 1] = '\0';
    }
  };
  try {
    f();
    put("");
    return QFLEX_GB300_OK;
  } catch (const std::string& e) {
    put(e);
    return QFLEX_GB300_ERR_INPUT;
  } catch (const std::bad_alloc&) {
    put("ERROR (qflex_gb300) --> host allocation failed");
    return QFLEX_GB300_ERR_ARG;
  } catch (const std::exception& e) {
    put(e.what());
    return QFLEX_GB300_ERR_INPUT;
  } catch (...) {  // nothing may cross the C ABI
    put("ERROR (qflex_gb300) --> unknown exception");
    return QFLEX_GB300_ERR_INPUT;
  }
}

}  // namespace

extern "C" {

int qflex_gb300_circuit_load(const char* text, qflex_gb300_circuit** out, char* err, size_t err_len) {
  if (!out) return QFLEX_GB300_ERR_ARG;
  *out = nullptr;
  std::unique_ptr<qflex_gb300_circuit> c;
  const int rc = parse_guarded(err, err_len, [&] {
    c = std::make_unique<qflex_gb300_circuit>();
    c->circuit.load(text ? text : "");
  });
  if (rc == QFLEX_GB300_OK) *out = c.release();
  return rc;
}

void qflex_gb300_circuit_free(qflex_gb300_circuit* circuit) { delete circuit; }

size_t qflex_gb300_circuit_num_active_qubits(const qflex_gb300_circuit* c) {
  return c ? (size_t)c->circuit.num_active_qubits : 0;
}

size_t qflex_gb300_circuit_depth(const qflex_gb300_circuit* c) { return c ? (size_t)c->circuit.depth : 0; }

size_t qflex_gb300_circuit_gate_count(const qflex_gb300_circuit* c) { return c ? c->circuit.gates.size() : 0; }

int qflex_gb300_circuit_gate(const qflex_gb300_circuit* c, size_t i, const char** name, const char** raw,
                             size_t* cycle, size_t* qubits, size_t qubits_cap, size_t* n_qubits, double* params,
                             size_t params_cap, size_t* n_params) {
  if (!c || i >= c->circuit.gates.size()) return QFLEX_GB300_ERR_ARG;
  const qfx::Gate& g = c->circuit.gates[i];
  if (name) *name = g.name.c_str();
  if (raw) *raw = g.raw.c_str();
  if (cycle) *cycle = (size_t)g.cycle;
  for (size_t q = 0; q < g.qubits.size() && q < qubits_cap && qubits; ++q) qubits[q] = (size_t)g.qubits[q];
  if (n_qubits) *n_qubits = g.qubits.size();
  for (size_t q = 0; q < g.params.size() && q < params_cap && params; ++q) params[q] = g.params[q];
  if (n_params) *n_params = g.params.size();
  return QFLEX_GB300_OK;
}

int qflex_gb300_grid_load(const char* text, size_t* I, size_t* J, size_t* off, size_t off_cap, size_t* n_off,
                          char* err, size_t err_len) {
  return parse_guarded(err, err_len, [&] {
    qfx::Grid g;
    g.load(text ? text : "");
    if (I) *I = (size_t)g.I;
    if (J) *J = (size_t)g.J;
    for (size_t q = 0; q < g.qubits_off.size() && q < off_cap && off; ++q) {
      off[2 * q] = (size_t)g.qubits_off[q].first;
      off[2 * q + 1] = (size_t)g.qubits_off[q].second;
    }
    if (n_off) *n_off = g.qubits_off.size();
  });
}

int qflex_gb300_ordering_load(const char* text, char* out, size_t cap, size_t* n_instructions, size_t* needed,
                              char* err, size_t err_len) {
  return parse_guarded(err, err_len, [&] {
    qfx::Ordering o;
    o.load(text ? text : "");
    std::string joined;
    for (size_t i = 0; i < o.instructions.size(); ++i) {
      if (i) joined += '\n';
      joined += o.instructions[i];
    }
    if (n_instructions) *n_instructions = o.instructions.size();
    if (needed) *needed = joined.size() + 1;
    if (out && cap) {
      const size_t n = std::min(cap - 1, joined.size());
      std::memcpy(out, joined.data(), n);
      out[n] = '\0';
    }
  });
}

int qflex_gb300_synchronize(qflex_gb300_context* ctx) {
  return guarded(ctx, [&] {
    if (!ctx->engine) throw QFX_ERR("context has no engine");
    cudaError_t e = cudaStreamSynchronize(ctx->engine->stream());
    if (e != cudaSuccess) throw qfx::cuda_error_string(e, "cudaStreamSynchronize");
    // A tensor-core product queued by qflex_gb300_multiply reports an
    // expired pipeline wait here.
    if (ctx->engine->has_error_flag()) ctx->engine->check_error_flag();
  });
}

}  // extern "C"

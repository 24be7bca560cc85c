// Symbolic execution of the reference's contraction recursion
// (src/contraction_utils.cpp:16-354 and multiply, src/tensor.cpp:1045-1194)
// on index metadata, recording a static device program.
//
// Storage model. Every device buffer is written once (by a permute or a
// GEMM) and is immutable afterwards, so tensors may share buffers freely:
// a projected cut slice is a view into its parent, a merge into an empty
// patch shares the source's buffer, and the reference's in-place reorder
// becomes "permute into a fresh buffer, release the old one". Buffers are
// recycled through power-of-two size classes (every dimension in these
// networks is a power of two), so the arena stays at the live-set maximum.
#include "planner.h"

#include <algorithm>
#include <map>
#include <set>
#include <unordered_map>
#include <unordered_set>

namespace qfx {
namespace {

constexpr std::size_t kLeafMark = std::size_t(1) << 62;

int ilog2_exact(std::size_t v) {
  int l = 0;
  while ((std::size_t(1) << l) < v) ++l;
  if ((std::size_t(1) << l) != v)
    throw QFX_ERR("Dimension ", v, " is not a power of two.");
  return l;
}

std::vector<std::string> minus(const std::vector<std::string>& v, const std::vector<std::string>& w) {
  std::vector<std::string> out;
  for (const auto& x : v)
    if (std::find(w.begin(), w.end(), x) == w.end()) out.push_back(x);
  return out;
}

std::vector<std::string> common_of(const std::vector<std::string>& v,
                                   const std::vector<std::string>& w) {
  std::vector<std::string> out;
  for (const auto& x : v)
    if (std::find(w.begin(), w.end(), x) != w.end()) out.push_back(x);
  return out;
}

std::vector<std::string> concat(std::vector<std::string> a, const std::vector<std::string>& b) {
  a.insert(a.end(), b.begin(), b.end());
  return a;
}

// A tensor during planning. `idx`/`dim` mirror the reference's index order
// (its in-place reorders decide its error messages); `phys`/`pdim` are the
// order the data actually has in its buffer, which the planner changes only
// when a product or a projection needs another layout.
struct STensor {
  std::vector<std::string> idx;
  std::vector<std::size_t> dim;
  std::vector<std::string> phys;
  std::vector<std::size_t> pdim;
  int buf = -1;
  std::size_t off = 0;
  std::size_t size() const {
    std::size_t s = 1;
    for (auto d : dim) s *= d;
    return s;
  }
  std::size_t dim_of(const std::string& name) const {
    auto it = std::find(idx.begin(), idx.end(), name);
    return dim[it - idx.begin()];
  }
  std::string describe() const {
    std::string s = cat("Tensor of rank ", idx.size(), ": ");
    for (std::size_t i = 0; i < idx.size(); ++i)
      s += cat(idx[i], " -> ", dim[i], i + 1 < idx.size() ? ", " : "");
    return s;
  }
};

// The reference's scratch plan and memory-limit check
// (ContractionData::Initialize, src/contraction_utils.cpp:30-155).
double reference_plan_bytes(const Network& net, const std::vector<Op>& ops) {
  std::unordered_map<std::string, std::size_t> dim;
  std::map<Coord, std::vector<std::string>> gidx;
  std::map<Coord, std::size_t> gsize;
  for (const auto& col : net.columns) {
    gidx[col.pos] = col.indices;
    std::size_t s = 1;
    for (std::size_t i = 0; i < col.indices.size(); ++i) {
      dim[col.indices[i]] = col.dims[i];
      s *= col.dims[i];
    }
    gsize[col.pos] = s;
  }
  std::unordered_map<std::string, std::vector<std::string>> pidx;
  std::unordered_map<std::string, std::size_t> pmax, cut_copy;
  auto symdiff = [](const std::vector<std::string>& a, const std::vector<std::string>& b) {
    return concat(minus(a, b), minus(b, a));
  };
  auto grow = [&](const std::string& p) {
    std::size_t s = 1;
    for (const auto& x : pidx[p]) s *= dim.at(x);
    pmax[p] = std::max(pmax[p], s);
  };
  for (const auto& op : ops) {
    if (op.kind == Op::EXPAND) {
      pidx[op.patch] = symdiff(pidx[op.patch], gidx[op.tensor]);
      grow(op.patch);
    } else if (op.kind == Op::CUT) {
      const std::string name = cut_index_name(op);
      for (std::size_t side = 0; side < op.tensors.size(); ++side) {
        auto& v = gidx[op.tensors[side]];
        v = minus(v, {name});
        cut_copy[cat("cut-", name, ":size-", side)] = gsize[op.tensors[side]];
      }
    } else {
      pidx[op.target] = symdiff(pidx[op.target], pidx[op.source]);
      grow(op.target);
    }
  }
  std::size_t max_size = 0, total = 0;
  std::unordered_set<std::size_t> unique;
  for (auto& [p, s] : pmax) {
    max_size = std::max(max_size, s);
    unique.insert(s);
    total += s;
  }
  total += max_size;
  for (auto s : unique) total += s;
  for (auto& [n, s] : cut_copy) total += s;
  return double(total) * 8.0;
}

class Planner {
 public:
  Planner(const Network& net, const std::vector<Op>& ops, std::size_t n_amps,
          std::function<bool(std::size_t, std::size_t, std::size_t)> b_kmajor, bool open_terminals)
      : net_(net), ops_(ops), b_kmajor_(std::move(b_kmajor)) {
    prog_.n_amplitudes = n_amps;
    // Terminal cuts stay open indices when every one of them takes all its
    // values and no two-qubit cut follows the first of them: the ops after
    // them then run once on tensors that carry the open (o) indices, and
    // the final tensor holds all the region's amplitudes, instead of the
    // reference's re-run of those ops per terminal value
    // (src/contraction_utils.cpp:300-314).
    open_ = open_terminals;
    bool seen_terminal = false;
    for (const auto& op : ops_) {
      if (op.kind != Op::CUT) continue;
      if (op.tensors.size() == 1) {
        seen_terminal = true;
        if (!op.values.empty()) {
          bool full = op.values.size() == 2;
          for (std::size_t v = 0; v < op.values.size() && full; ++v) full = op.values[v] == v;
          if (!full) open_ = false;
        }
        open_order_.push_back(cut_index_name(op));
      } else if (seen_terminal) {
        open_ = false;
      }
    }
    if (open_order_.empty()) open_ = false;
  }

  Program run() {
    // Grid tensors are allocated first and never recycled.
    prog_.column_offset.resize(net_.columns.size());
    for (std::size_t c = 0; c < net_.columns.size(); ++c) {
      const auto& col = net_.columns[c];
      STensor t{col.indices, col.dims, col.indices, col.dims, -1, 0};
      t.buf = alloc(t.size());
      prog_.column_offset[c] = bufs_[t.buf].off;
      grid_[col.pos] = t;
    }
    std::unordered_map<std::string, bool> active;
    contract(0, 0, active);
    prog_.results_offset = top_;
    prog_.n_leaves = leaves_;
    prog_.arena_elems = top_ + round_up(std::max<std::size_t>(leaves_, 1));
    for (auto& op : prog_.ops)
      if (op.c >= kLeafMark) op.c = prog_.results_offset + (op.c - kLeafMark);
    for (auto& [key, idx] : shape_index_) prog_.shapes[idx].count = shape_count_[idx];
    return std::move(prog_);
  }

 private:
  static std::size_t round_up(std::size_t n) { return (n + 31) / 32 * 32; }

  int alloc(std::size_t n) {
    const int cls = ilog2_exact(std::max<std::size_t>(n, 32));
    auto& fl = free_[cls];
    int b;
    if (!fl.empty()) {
      b = fl.back();
      fl.pop_back();
    } else {
      b = (int)bufs_.size();
      bufs_.push_back(Buf{top_, cls, 0});
      top_ += std::size_t(1) << cls;
    }
    bufs_[b].refs = 1;
    return b;
  }
  void incref(int b) {
    if (b >= 0) ++bufs_[b].refs;
  }
  void decref(int b) {
    if (b >= 0 && --bufs_[b].refs == 0) free_[bufs_[b].cls].push_back(b);
  }
  // dst = src with reference counting.
  void assign(STensor& dst, const STensor& src) {
    incref(src.buf);
    decref(dst.buf);
    dst = src;
  }
  std::size_t addr(const STensor& t) const { return bufs_[t.buf].off + t.off; }

  // Tensor::reorder (src/tensor.cpp:866-911): the reference's index order
  // changes; the data is moved only when physical() asks for it.
  static void reorder(STensor& t, const std::vector<std::string>& order) {
    if (order == t.idx) return;
    std::vector<std::size_t> nd(order.size());
    for (std::size_t p = 0; p < order.size(); ++p) nd[p] = t.dim_of(order[p]);
    t.idx = order;
    t.dim = nd;
  }

  // Moves the data of `t` into index order `order` (an out-of-place
  // permute into a fresh buffer) unless it is already laid out that way.
  void physical(STensor& t, const std::vector<std::string>& order, std::size_t leaf_dst = 0) {
    if (order.empty() && t.phys.empty()) return;
    if (order == t.phys) return;
    const std::size_t r = t.phys.size();
    std::vector<int> lg(r);
    for (std::size_t i = 0; i < r; ++i) lg[i] = ilog2_exact(t.pdim[i]);
    std::vector<int> s_old(r, 0);
    for (std::size_t i = r; i-- > 1;) s_old[i - 1] = s_old[i] + lg[i];
    std::vector<std::size_t> new_pos(r);
    std::vector<std::size_t> new_dim(r);
    for (std::size_t i = 0; i < r; ++i) {
      new_pos[i] = std::find(order.begin(), order.end(), t.phys[i]) - order.begin();
      new_dim[new_pos[i]] = t.pdim[i];
    }
    std::vector<int> s_new(r, 0);
    for (std::size_t p = r; p-- > 1;) s_new[p - 1] = s_new[p] + ilog2_exact(new_dim[p]);
    DevOp op{DevOp::PERMUTE};
    int nbits = 0;
    for (std::size_t i = 0; i < r; ++i) nbits += lg[i];
    if (nbits > 40) throw QFX_ERR("Tensor of 2^", nbits, " elements is too large.");
    op.nbits = nbits;
    for (std::size_t i = 0; i < r; ++i)
      for (int b = 0; b < lg[i]; ++b) op.perm[s_old[i] + b] = (std::uint8_t)(s_new[new_pos[i]] + b);
    bool identity = true;
    for (int b = 0; b < nbits; ++b) identity &= (op.perm[b] == b);
    if (!identity) {
      const int nb = leaf_dst ? -1 : alloc(t.size());
      op.a = addr(t);
      op.c = leaf_dst ? leaf_dst : bufs_[nb].off;
      prog_.permute_bytes += 16.0 * double(t.size());
      prog_.ops.push_back(op);
      decref(t.buf);
      t.buf = nb;
      t.off = 0;
    }
    t.phys = order;
    t.pdim = new_dim;
  }

  // multiply (src/tensor.cpp:1045-1194): C(left, right) = A(left, common) *
  // B(common, right); A and B are reordered "in place".
  STensor multiply(STensor& A, STensor& B) {
    const auto left = minus(A.idx, B.idx);
    const auto right = minus(B.idx, A.idx);
    const auto common = common_of(A.idx, B.idx);
    std::size_t m = 1, n = 1, k = 1;
    for (const auto& x : left) m *= A.dim_of(x);
    for (const auto& x : right) n *= B.dim_of(x);
    for (std::size_t i = 0; i < common.size(); ++i) {
      const std::size_t da = A.dim_of(common[i]), db = B.dim_of(common[i]);
      if (da != db)
        throw QFX_ERR("Common indices must have matching dimensions, but at index: ", i,
                      ", the dimensions are A: ", da, ", B: ", db, ".");
      k *= da;
    }
    reorder(A, concat(left, common));
    reorder(B, concat(common, right));
    // Tensor-core products read B as (right, common) rows (K-major); the
    // CUDA-core kernels read the reference's (common, right) layout.
    const bool b_nk = b_kmajor_(m, n, k);
    physical(A, concat(left, common));
    physical(B, b_nk ? concat(right, common) : concat(common, right));
    STensor C;
    C.idx = concat(left, right);
    for (const auto& x : left) C.dim.push_back(A.dim_of(x));
    for (const auto& x : right) C.dim.push_back(B.dim_of(x));
    C.phys = C.idx;
    C.pdim = C.dim;
    C.buf = alloc(m * n);
    DevOp op{DevOp::GEMM};
    op.a = addr(A);
    op.b = addr(B);
    op.c = bufs_[C.buf].off;
    op.m = m;
    op.n = n;
    op.k = k;
    op.b_nk = b_nk;
    const auto key = std::make_tuple(m, n, k);
    auto it = shape_index_.find(key);
    if (it == shape_index_.end()) {
      it = shape_index_.emplace(key, (int)prog_.shapes.size()).first;
      prog_.shapes.push_back(GemmShape{m, n, k, 0});
      shape_count_.push_back(0);
    }
    op.shape_id = it->second;
    ++shape_count_[it->second];
    prog_.gemm_flop += 8.0 * double(m) * double(n) * double(k);
    prog_.ops.push_back(op);
    return C;
  }

  // ContractionData::ContractGrid (src/contraction_utils.cpp:223-354).
  void contract(std::size_t pos, std::size_t out_idx, std::unordered_map<std::string, bool> active) {
    bool have_output = false;
    STensor output;
    std::size_t output_op = 0;
    // Grid tensors of open terminal cuts, restored when this slice is done
    // (the products after the cut reorder them in place, as the reference
    // reorders its projected copies).
    std::vector<std::pair<Coord, STensor>> saved;
    auto restore = [&]() {
      for (auto& [pos_, t] : saved) {
        assign(grid_.at(pos_), t);
        decref(t.buf);
      }
      saved.clear();
    };
    while (pos < ops_.size()) {
      const Op& op = ops_[pos++];
      const bool last = pos == ops_.size();
      if (op.kind == Op::EXPAND) {
        STensor& next = grid_.at(op.tensor);
        if (!active[op.patch]) {
          assign(scratch_[op.patch], next);
          active[op.patch] = true;
          continue;
        }
        STensor result = multiply(scratch_[op.patch], next);
        if (last) {
          output = result;
          have_output = true;
          output_op = prog_.ops.size() - 1;
          continue;
        }
        decref(scratch_[op.patch].buf);
        scratch_[op.patch] = result;
      } else if (op.kind == Op::CUT) {
        const std::string index = cut_index_name(op);
        STensor& ta = grid_.at(op.tensors[0]);
        if (open_ && op.tensors.size() == 1) {
          // Open terminal index: the checks of the projection, no
          // projection; the index stays on the tensor for the ops after it.
          if (std::find(ta.idx.begin(), ta.idx.end(), index) == ta.idx.end())
            throw QFX_ERR("Index ", index, " is not an index of the tensor at (", op.tensors[0].first, ",",
                          op.tensors[0].second, ").");
          if (index != ta.idx[0])
            throw QFX_ERR("Failed to call project(). Error:\n\t[Index: '", index,
                          "' has to be equal to indices[0]: '", ta.idx[0], "'.]");
          out_idx *= op.values.empty() ? ta.dim_of(index) : op.values.size();
          saved.emplace_back(op.tensors[0], STensor{});
          assign(saved.back().second, ta);
          continue;
        }
        STensor copy_a;
        assign(copy_a, ta);
        lead_with(copy_a, index);
        std::vector<std::size_t> values = op.values;
        if (values.empty()) {
          if (std::find(copy_a.idx.begin(), copy_a.idx.end(), index) == copy_a.idx.end())
            throw QFX_ERR("Index ", index, " is not an index of the tensor at (",
                          op.tensors[0].first, ",", op.tensors[0].second, ").");
          for (std::size_t v = 0; v < copy_a.dim_of(index); ++v) values.push_back(v);
        }
        if (op.tensors.size() > 1) {
          STensor& tb = grid_.at(op.tensors[1]);
          STensor copy_b;
          assign(copy_b, tb);
          lead_with(copy_b, index);
          for (std::size_t v : values) {
            project(copy_a, index, v, grid_.at(op.tensors[0]));
            project(copy_b, index, v, grid_.at(op.tensors[1]));
            contract(pos, out_idx, active);
          }
          assign(grid_.at(op.tensors[1]), copy_b);
          decref(copy_b.buf);
        } else {
          out_idx *= values.size();
          for (std::size_t v : values) {
            project(copy_a, index, v, grid_.at(op.tensors[0]));
            contract(pos, out_idx, active);
            ++out_idx;
          }
        }
        assign(grid_.at(op.tensors[0]), copy_a);
        decref(copy_a.buf);
        return;
      } else {
        if (!active[op.target]) {
          assign(scratch_[op.target], scratch_[op.source]);
          active[op.target] = true;
          continue;
        }
        STensor result = multiply(scratch_[op.source], scratch_[op.target]);
        if (last) {
          output = result;
          have_output = true;
          output_op = prog_.ops.size() - 1;
          continue;
        }
        decref(scratch_[op.target].buf);
        scratch_[op.target] = result;
      }
    }
    if (!have_output)
      throw QFX_ERR("Contraction did not complete; the ordering does not end with a product.");
    if (open_) {
      // The final tensor carries the open terminal indices: lay it out in
      // cut order (first cut most significant, as the output states are
      // numbered) straight into the results region.
      std::vector<std::string> sorted_idx = output.idx, sorted_open = open_order_;
      std::sort(sorted_idx.begin(), sorted_idx.end());
      std::sort(sorted_open.begin(), sorted_open.end());
      if (sorted_idx != sorted_open)
        throw QFX_ERR("Contraction did not complete; final tensor is: ", output.describe());
      const std::size_t count = output.size();
      if (out_idx + count > prog_.n_amplitudes)
        throw QFX_ERR("Output index ", out_idx + count - 1, " exceeds the ", prog_.n_amplitudes,
                      " output states.");
      if (output.phys == open_order_)
        prog_.ops[output_op].c = kLeafMark + leaves_;
      else
        physical(output, open_order_, kLeafMark + leaves_);
      for (std::size_t v = 0; v < count; ++v) prog_.leaf_amp.push_back((std::uint32_t)(out_idx + v));
      leaves_ += count;
      decref(output.buf);
      restore();
      return;
    }
    if (output.size() != 1)
      throw QFX_ERR("Contraction did not complete; final tensor is: ", output.describe());
    if (out_idx >= prog_.n_amplitudes)
      throw QFX_ERR("Output index ", out_idx, " exceeds the ", prog_.n_amplitudes,
                    " output states.");
    prog_.ops[output_op].c = kLeafMark + leaves_;
    prog_.leaf_amp.push_back((std::uint32_t)out_idx);
    ++leaves_;
    decref(output.buf);
  }

  // Tensor::project (src/tensor.cpp:280-316): a view of one slice of the
  // leading index.
  void project(const STensor& src, const std::string& index, std::size_t value, STensor& dst) {
    if (src.idx.empty() || index != src.idx[0])
      throw QFX_ERR("Failed to call project(). Error:\n\t[Index: '", index,
                    "' has to be equal to indices[0]: '", src.idx.empty() ? "" : src.idx[0],
                    "'.]");
    if (value >= src.dim[0])
      throw QFX_ERR("Failed to call project(). Error:\n\t[index_value: ", value,
                    " must be contained in [0, ", src.dim[0], ").]");
    if (src.phys.empty() || src.phys[0] != index)
      throw QFX_ERR("Projected index ", index, " is not leading in memory.");
    STensor view;
    view.idx.assign(src.idx.begin() + 1, src.idx.end());
    view.dim.assign(src.dim.begin() + 1, src.dim.end());
    view.phys.assign(src.phys.begin() + 1, src.phys.end());
    view.pdim.assign(src.pdim.begin() + 1, src.pdim.end());
    view.buf = src.buf;
    view.off = src.off + value * (src.size() / src.dim[0]);
    assign(dst, view);
  }

  // Makes the cut index leading in memory when it leads the reference's
  // order but not the buffer (after a tensor-core layout of the tensor).
  void lead_with(STensor& t, const std::string& index) {
    if (t.idx.empty() || t.idx[0] != index || t.phys[0] == index) return;
    std::vector<std::string> order{index};
    for (const auto& x : t.phys)
      if (x != index) order.push_back(x);
    physical(t, order);
  }

  struct Buf {
    std::size_t off;
    int cls;
    int refs;
  };
  const Network& net_;
  const std::vector<Op>& ops_;
  std::function<bool(std::size_t, std::size_t, std::size_t)> b_kmajor_;
  Program prog_;
  std::vector<Buf> bufs_;
  std::vector<int> free_[64];
  std::size_t top_ = 0;
  std::size_t leaves_ = 0;
  bool open_ = false;                    // terminal cuts kept as open indices
  std::vector<std::string> open_order_;  // their index names in cut order
  std::map<Coord, STensor> grid_;
  std::unordered_map<std::string, STensor> scratch_;
  std::map<std::tuple<std::size_t, std::size_t, std::size_t>, int> shape_index_;
  std::vector<std::size_t> shape_count_;
};

}  // namespace

Program plan_contraction(const Network& net, const std::vector<Op>& ops, std::size_t n_amplitudes,
                         double memory_limit,
                         std::function<bool(std::size_t, std::size_t, std::size_t)> b_kmajor,
                         bool open_terminals) {
  const double ref_bytes = reference_plan_bytes(net, ops);
  if (ref_bytes > memory_limit)
    throw QFX_ERR("Failed to call Initialize(). Error:\n\t[Required space (",
                  readable_memory_string(ref_bytes), ") exceeds memory limit (",
                  readable_memory_string(memory_limit), "). Cancelling simulation.]");
  if (!b_kmajor) b_kmajor = [](std::size_t, std::size_t, std::size_t) { return false; };
  Planner p(net, ops, n_amplitudes, std::move(b_kmajor), open_terminals);
  Program prog = p.run();
  prog.reference_bytes = ref_bytes;
  return prog;
}

}  // namespace qfx

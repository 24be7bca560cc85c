// Complex64 products on the sm_103a tensor cores (tcgen05 + TMEM + TMA),
// split precision.
//
// C = A * B with A (m x k) and B given as Bt (n x k), both K-major complex64.
// Each complex operand is split into four real planes -- re_hi, re_lo,
// im_hi, im_lo -- with x = hi + lo, hi and lo exactly representable in
// TF32 (round-to-nearest), so x is carried to ~22 significant bits. The
// product keeps the three leading terms of every real product
// (hi*hi + hi*lo + lo*hi) and the complex product uses four real products:
//   C_re = Ar Br - Ai Bi,   C_im = Ar Bi + Ai Br,
// i.e. 12 TF32 MMAs per k-step. The minus sign is the instruction
// descriptor's negate-A bit. The 3xFP16 kind (below) instead keeps a
// negated copy of Bt's imaginary planes so that one N = 256 MMA yields C_re
// and C_im side by side: 6 MMAs per k-step, each twice as large.
//
// Accumulation. The tensor core accumulates in FP32 but rounds toward zero,
// so a long sum in one TMEM accumulator drifts in proportion to the number
// of k-steps (measured: 6e-5 relative error at k = 4096). The k range is
// therefore cut into chunks of CHUNK k-steps; chunk c accumulates from zero
// in TMEM buffer c % 2 (C_re and C_im, 2 x BN columns) while the epilogue
// warps add chunk c - 1 into FP32 registers with round-to-nearest. The
// result is as accurate as FP32 CUDA-core arithmetic.
//
// Kernel structure (persistent, one CTA per SM taking 128 x 128 complex
// output tiles in turn, 320 threads):
//   warp 0      TMA producer: 4-D boxes bring one k-step of the operands'
//               planes per stage (3xTF32 / BF16x3: all planes of a row in
//               one 128-byte row; 3xFP16: A's 128-byte rows and three
//               blocks of 64-byte B rows, see umma_f16_kstep)
//   warp 1      TMEM allocation and the single MMA-issuing thread, whose
//               instruction stream paces the tensor core: its loops count
//               stages and chunks instead of dividing, and a barrier test
//               reads no timer unless it must wait
//   warps 2..9  epilogue: warp w owns TMEM lanes 32 (w % 4) .. + 31 and one
//               half of the columns; it drains every chunk into registers
//               and finally stores complex64 tiles with TMA bulk stores
// Every mbarrier wait is bounded in time; on expiry the CTA records an
// error code, stops issuing work, waits (bounded) for what it issued and
// frees its TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "kernels.h"
#include "tc_gemm.h"

namespace qfx {
namespace {

constexpr int BM = 128, BN = 128, BK = 8;
constexpr int STAGES = 5;
// One k-step of an operand tile: every row holds the four planes' 8 values
// side by side (4 x 32 bytes = one 128-byte row in the 128-byte swizzle),
// so plane p is the K-major matrix starting 32 p bytes into the tile.
constexpr int TILE_A = BM * 128;
constexpr int TILE_B = BN * 128;
constexpr int STAGE_BYTES = TILE_A + TILE_B;
// 3xFP16 stage: 40 KB of five 8 KB blocks, one k-step: A's 128 rows of 128
// bytes (re hi, lo, im hi, lo; 128-byte swizzle) fill the first two, then B
// rows of 64 bytes (hi, lo; 64-byte swizzle) of -im, re and im. (The CTA
// pair loads A's re and im halves as separate 64-byte blocks instead.)
constexpr int F16_BLOCK = BM * 64;
constexpr int F16_STAGE_BYTES = 5 * F16_BLOCK;
constexpr int EPI_WARPS = 8;
constexpr int TMEM_COLS = 4 * BN;         // two chunk buffers of (re, im)
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int STAGING_BYTES = 8 * 32 * 32 * 8;  // 32 x 32 complex64 per epilogue warp
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + STAGING_BYTES + 1024 + 256;
// The deep 3xFP16 variant: five stages and a 2 KB output box per epilogue
// warp (32 rows x 8 complex, 64-byte swizzle).
constexpr int DEEP_STAGES = 5;
constexpr int DEEP_STAGING_BYTES = EPI_WARPS * 2048;
constexpr int DEEP_SMEM_BYTES = DEEP_STAGES * F16_STAGE_BYTES + DEEP_STAGING_BYTES + 1024 + 256;
// The wide 3xFP16 variant: 16 epilogue warps, four per TMEM lane quadrant,
// each draining a quarter of the tile's columns (the chunk drain is the
// critical path when chunks are one k-step long); one 4 KB output slot per
// warp in the same staging area. Needs the bulk-store output map.
constexpr int WIDE_EPI_WARPS = 16;
constexpr int WIDE_THREADS = 64 + 32 * WIDE_EPI_WARPS;
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ std::uint32_t smem_u32(const void* p) {
  return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(std::uint64_t* bar, std::uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(std::uint64_t* bar, std::uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(std::uint64_t* bar, std::uint32_t parity) {
  std::uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Limit of a pipeline wait: the 64-bit value the host keeps after the error
// code in the error-flag buffer (err[2..3], written when the buffer is
// created and by the "tc_wait_ns" option), or WAIT_NS when it is 0. Read
// only once a wait has to spin. The drains on the abort path keep WAIT_NS.
__device__ __forceinline__ unsigned long long wait_limit_ns(const int* err) {
  const unsigned long long v = *reinterpret_cast<const volatile unsigned long long*>(err + 2);
  return v ? v : WAIT_NS;
}
// Bounded wait: false (and an error code) when the phase does not complete
// within the wait limit or another warp of the CTA has already given up.
__device__ __forceinline__ bool mbar_wait(std::uint64_t* bar, std::uint32_t parity, volatile int* abort_flag,
                                          int* err, int code) {
  if (mbar_test(bar, parity)) return true;  // the common case reads no timer
  const unsigned long long t0 = now_ns(), limit = wait_limit_ns(err);
  while (!mbar_test(bar, parity)) {
    if (*abort_flag) return false;
    if (now_ns() - t0 > limit) {
      *abort_flag = 1;
      atomicExch(err, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_4d(const CUtensorMap* map, std::uint64_t* bar, void* dst, int c0,
                                            int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<std::uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Bulk tensor store of a shared-memory box to global memory (C tiles), its
// commit group, and the waits for the box's shared-memory reads / for the
// global writes to finish.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<std::uint64_t>(map)),
               "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// v * 2^e, exact unless the result leaves the normal range (then rounded
// like ldexpf): a multiply by the power of two when 2^e is a normal float.
__device__ __forceinline__ float scale2(float v, int e) {
  return (e >= -126 && e <= 127) ? v * __uint_as_float(std::uint32_t(e + 127) << 23) : ldexpf(v, e);
}

// Shared-memory matrix descriptor: K-major operand inside rows of 128 bytes
// in the 128-byte swizzle (the start address may sit 32, 64 or 96 bytes into
// the row, as for a K offset), 8-row groups 1024 bytes apart.
__device__ __forceinline__ std::uint64_t smem_desc_sw128(std::uint32_t addr) {
  std::uint64_t d = 0;
  d |= std::uint64_t((addr & 0x3FFFF) >> 4);       // start address
  d |= std::uint64_t(1) << 16;                     // leading byte offset (unused here)
  d |= std::uint64_t(1024 >> 4) << 32;             // stride byte offset
  d |= std::uint64_t(1) << 46;                     // descriptor version
  d |= std::uint64_t(2) << 61;                     // 128-byte swizzle
  return d;
}

// The same for rows of 64 bytes in the 64-byte swizzle (8-row groups 512
// bytes apart); the BF16x3 kernel keeps its third pieces there.
__device__ __forceinline__ std::uint64_t smem_desc_sw64(std::uint32_t addr) {
  std::uint64_t d = 0;
  d |= std::uint64_t((addr & 0x3FFFF) >> 4);
  d |= std::uint64_t(1) << 16;
  d |= std::uint64_t(512 >> 4) << 32;
  d |= std::uint64_t(1) << 46;
  d |= std::uint64_t(4) << 61;                     // 64-byte swizzle
  return d;
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr std::uint32_t idesc_tf32(int m, int n, bool negate_a) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (negate_a ? (1u << 13) : 0u) |
         (std::uint32_t(n >> 3) << 17) | (std::uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b,
                                          std::uint32_t idesc, std::uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
// Instruction descriptor, kind::f16 with FP16 A and B (format 0), F32 D.
__host__ __device__ constexpr std::uint32_t idesc_f16(int m, int n, bool negate_a) {
  return (1u << 4) | (negate_a ? (1u << 13) : 0u) | (std::uint32_t(n >> 3) << 17) | (std::uint32_t(m >> 4) << 24);
}
__device__ __forceinline__ void umma_f16(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b, std::uint32_t idesc,
                                         std::uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
// One k-step of the 3xFP16 product (six M = 128, N = 256 MMAs, small terms
// first) in one instruction block. The stage is A's 16 KB block of 128-byte
// rows (re hi, lo, im hi, lo; 128-byte swizzle, high descriptor word `hia`)
// and B's 8 KB blocks of 64-byte rows (-im, re, im; 64-byte swizzle, `hib`).
// The low descriptor words differ from `lo` (A re hi) by fixed offsets in
// 16-byte units: A re lo +2, A im hi +4, lo +6; B -im +1024, +1026, B re
// +1536, +1538. `acc` = 0 starts the accumulator.
__device__ __forceinline__ void umma_f16_kstep(std::uint32_t d, std::uint32_t lo, std::uint32_t hia,
                                               std::uint32_t hib, std::uint32_t idesc, std::uint32_t acc,
                                               std::uint32_t bstep = 512) {
  // bstep: distance from the -Bi block to the Br block in 16-byte units
  // (rows of the tile x 64 bytes / 16).
  asm volatile(
      "{\n .reg .pred p0, p1;\n .reg .b32 l1, l2, l3, l4, l5, l6, l7;\n"
      " .reg .b64 arh, arl, aih, ail, b2h, b2l, b1h, b1l;\n"
      " setp.ne.b32 p0, %5, 0;\n setp.eq.b32 p1, %5, %5;\n"
      " add.u32 l1, %1, 2;\n add.u32 l2, %1, 4;\n add.u32 l3, %1, 6;\n add.u32 l4, %1, 1024;\n"
      " add.u32 l5, %1, 1026;\n add.u32 l6, l4, %6;\n add.u32 l7, l6, 2;\n"
      " mov.b64 arh, {%1, %2};\n mov.b64 arl, {l1, %2};\n mov.b64 aih, {l2, %2};\n mov.b64 ail, {l3, %2};\n"
      " mov.b64 b2h, {l4, %3};\n mov.b64 b2l, {l5, %3};\n mov.b64 b1h, {l6, %3};\n mov.b64 b1l, {l7, %3};\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], arh, b1l, %4, p0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], arl, b1h, %4, p1;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], aih, b2l, %4, p1;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], ail, b2h, %4, p1;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], arh, b1h, %4, p1;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], aih, b2h, %4, p1;\n}\n" ::"r"(d),
      "r"(lo), "r"(hia), "r"(hib), "r"(idesc), "r"(acc), "r"(bstep));
}

// Operand kinds of the single-CTA kernel: 3xTF32 planes (8 values of 4
// bytes per plane and k-step) or 3xFP16 planes (16 values of 2 bytes, rows
// scaled by powers of two).
// BF16x3: three BF16 pieces per value (x = b0 + b1 + b2 to ~24 bits).
enum SplitKind : int { KIND_TF32 = 0, KIND_FP16 = 1, KIND_BF16 = 2 };

// Compensation of the truncation bias. The tensor core's FP32 accumulation
// rounds toward zero, so every product comes out smaller by a fraction beta
// of itself that depends on the split kind and on how many k-steps a TMEM
// chunk accumulates (not on the shape). Measured on GB300 against complex128
// products of Gaussian operands (python -m qflex_gb300.kernel_bench bias), for
// chunks of one and two k-steps; other chunk lengths are not compensated.
// With err[1] != 0 (option "tc_debias") every output x becomes x + beta x,
// one fused multiply-add rounded to nearest (1 + beta itself is not a float:
// beta is below the float spacing at 1).
template <int KIND>
__device__ __forceinline__ float debias_beta(const int* err, int chunk, int kblocks) {
  if (*reinterpret_cast<const volatile int*>(err + 1) == 0) return 0.f;
  const int c = chunk < kblocks ? chunk : kblocks;
  if (c == 1) return KIND == KIND_FP16 ? 5.53e-8f : KIND == KIND_BF16 ? 4.47e-8f : 5.39e-8f;
  if (c == 2) return KIND == KIND_FP16 ? 1.535e-7f : KIND == KIND_BF16 ? 2.226e-7f : 1.52e-7f;
  return 0.f;
}
template <int KIND>
__device__ __forceinline__ void umma(std::uint32_t d, std::uint64_t a, std::uint64_t b, std::uint32_t id,
                                     std::uint32_t acc) {
  if (KIND == KIND_TF32)
    umma_tf32(d, a, b, id, acc);
  else
    umma_f16(d, a, b, id, acc);
}
// kind::f16 with BF16 A and B (format 1), F32 D.
__host__ __device__ constexpr std::uint32_t idesc_bf16(int m, int n, bool negate_a) {
  return idesc_f16(m, n, negate_a) | (1u << 7) | (1u << 10);
}
template <int KIND>
__host__ __device__ constexpr std::uint32_t idesc_kind(int m, int n, bool negate_a) {
  return KIND == KIND_TF32 ? idesc_tf32(m, n, negate_a)
                           : (KIND == KIND_FP16 ? idesc_f16(m, n, negate_a) : idesc_bf16(m, n, negate_a));
}

__device__ __forceinline__ void umma_commit(std::uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

#define TMEM_LD32(taddr, r)                                                                            \
  asm volatile(                                                                                        \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15," \
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                       \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),          \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),       \
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),    \
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),    \
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])                                            \
      : "r"(taddr))

#define TMEM_LD16(taddr, r)                                                                            \
  asm volatile(                                                                                        \
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),          \
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),       \
        "=r"(r[14]), "=r"(r[15])                                                                      \
      : "r"(taddr))

__device__ __forceinline__ void mbar_arrive(std::uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ---- Cluster (CTA pair) helpers ------------------------------------------------

__device__ __forceinline__ std::uint32_t cluster_rank() {
  std::uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Shared::cluster address of the same shared-memory offset in CTA `rank`.
__device__ __forceinline__ std::uint32_t peer_addr(const void* p, std::uint32_t rank) {
  std::uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test_cluster(std::uint64_t* bar, std::uint32_t parity) {
  std::uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_cluster(std::uint64_t* bar, std::uint32_t parity, volatile int* abort_flag,
                                                  int* err, int code) {
  if (mbar_test_cluster(bar, parity)) return true;
  const unsigned long long t0 = now_ns(), limit = wait_limit_ns(err);
  while (!mbar_test_cluster(bar, parity)) {
    if (*abort_flag) return false;
    if (now_ns() - t0 > limit) {
      *abort_flag = 1;
      atomicExch(err, code);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive_remote(std::uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
// TMA load into this CTA's shared memory that completes on a barrier of
// either CTA of the pair (`bar` is a shared::cluster address).
__device__ __forceinline__ void tma_load_4d_pair(const CUtensorMap* map, std::uint32_t bar, void* dst, int c0, int c1,
                                                 int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<std::uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void umma_tf32_pair(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b,
                                               std::uint32_t idesc, std::uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
// Commit of the issuing thread's MMAs, arriving on `bar` in both CTAs.
__device__ __forceinline__ void umma_commit_pair(std::uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(std::uint16_t(3))
      : "memory");
}

__device__ __forceinline__ void umma_f16_pair(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b,
                                              std::uint32_t idesc, std::uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// The single-CTA kernel body, persistent: CTA b takes output tiles b,
// b + gridDim.x, ... (grouped raster, batch entries after each other), and
// its producer, MMA issuer and epilogue run through the tiles on shared
// stage and chunk counters, so one tile's epilogue overlaps the next tile's
// loads and MMAs. KIND_FP16 operands carry power-of-two scale exponents
// (value = plane value * 2^-e) per row, or for A with a_blocks > 0 per 32
// values of a row (a_blocks = k / 32 per row; then every TMEM chunk, which
// lies inside one block, is scaled as it is added); the epilogue removes
// them. KIND_BF16 operands have
// six planes per k-step: b0, b1 of re and im in a 128-byte row (map_a /
// map_b) and b2 of re and im in a 64-byte row (map_a2 / map_b2).
//
// PAIR (3xFP16 only; a cluster of two CTAs, cta_group::2): a tile is 256
// rows x 128 complex columns. CTA r holds rows m0 + 128 r .. + 127 of A and
// the B rows of its half of the two N = 256 operands -- CTA 0 Br and -Bi,
// CTA 1 Bi and Br, so that (Br; Bi) and (-Bi; Br) are split across the pair
// at the same shared-memory offsets -- and one M = 256 MMA issued by CTA 0
// writes each CTA's 128 rows into that CTA's TMEM. Per SM and k-step that is
// 32 KB of operands instead of 40 KB, and half the MMA instructions.
// Synchronisation: both CTAs' TMA loads complete on CTA 0's full[s]; MMA
// commits are multicast to both CTAs (empty, acc_full, mma_done); both
// CTAs' epilogue warps arrive on CTA 0's acc_empty; cluster barriers after
// set-up and before TMEM is released.
//
// DEEP (3xFP16 single CTA): five stages instead of four; the output leaves
// in 2 KB boxes (32 rows x 8 complex) so that the staging area shrinks to
// 16 KB. Needs the bulk-store output map (tma_c).
//
// EPI (3xFP16 single CTA): epilogue warps, 8 (each drains half of the tile's
// columns, two 4 KB output slots) or 16 (a quarter, one slot; needs tma_c).
//
// TBN (3xFP16 single CTA): complex columns of a tile, 128 or 64. With 64 the
// MMAs are N = 128, a stage is 28 KB (five of them), and TMEM holds four
// chunk buffers instead of two, so the MMAs can run three chunks ahead of an
// epilogue that is storing a tile (products with a short k).
template <int KIND, bool PAIR = false, bool DEEP = false, int EPI = EPI_WARPS, int TBN = BN>
__device__ __forceinline__ void cgemm_split_body(const CUtensorMap* map_a, const CUtensorMap* map_b,
                                                 const CUtensorMap* map_a2, const CUtensorMap* map_b2,
                                                 const CUtensorMap* map_c, bool tma_c,
                                                 float2* __restrict__ C, int m, int n, int k, int batches,
                                                 std::uint64_t c_batch_stride, int* __restrict__ err, int CHUNK,
                                                 const int* __restrict__ exp_a,
                                                 const int* __restrict__ exp_b, int a_blocks) {
  constexpr int KSTEP = KIND == KIND_TF32 ? 8 : 16;  // k values per plane row of 32 bytes
  constexpr int TAIL = BM * 64;                       // BF16 third-piece tile of one operand
  constexpr bool NARROW = TBN != BN;
  constexpr int NST = KIND == KIND_BF16 ? 3 : (KIND == KIND_FP16 ? (PAIR || DEEP || NARROW ? 5 : 4) : STAGES);
  constexpr int F16_BBLOCK = TBN * 64;  // one B block: TBN rows of 64 bytes
  constexpr int SBYTES = KIND == KIND_BF16   ? 2 * (TILE_A + TAIL)
                         : KIND == KIND_FP16 ? (PAIR ? 4 * F16_BLOCK : 2 * F16_BLOCK + 3 * F16_BBLOCK)
                                             : STAGE_BYTES;
  constexpr int NBUF = TMEM_COLS / (2 * TBN);  // TMEM chunk buffers of (re, im)
  static_assert(!NARROW || (TBN == 64 && KIND == KIND_FP16 && !PAIR && !DEEP && EPI == EPI_WARPS),
                "the narrow tile is a single-CTA 3xFP16 kernel");
  static_assert(SBYTES % 1024 == 0, "stages keep the 1024-byte alignment of the 128-byte swizzle");
  constexpr int TM = PAIR ? 2 * BM : BM;  // rows of a tile
  constexpr int STAGE_REGION = DEEP ? DEEP_STAGES * F16_STAGE_BYTES : STAGES * STAGE_BYTES;
  constexpr int STG_BYTES = DEEP ? DEEP_STAGING_BYTES : STAGING_BYTES;
  static_assert(NST * SBYTES <= STAGE_REGION, "stages fit the shared memory of the launch");
  static_assert(!PAIR || KIND == KIND_FP16, "the CTA pair is a 3xFP16 kernel");
  static_assert(!DEEP || (KIND == KIND_FP16 && !PAIR), "the deep variant is a single-CTA 3xFP16 kernel");
  static_assert(EPI == EPI_WARPS || (EPI == WIDE_EPI_WARPS && KIND == KIND_FP16 && !PAIR && !DEEP),
                "16 epilogue warps: the single-CTA 3xFP16 kernel");
  constexpr int COLS = TBN * 4 / EPI;  // complex columns an epilogue warp drains and stores
  constexpr int SLOTS = STG_BYTES / EPI / 4096;  // 4 KB output slots per epilogue warp (DEEP: unused)
  extern __shared__ __align__(1024) std::uint8_t smem_raw[];
  std::uint8_t* smem = reinterpret_cast<std::uint8_t*>((reinterpret_cast<std::uintptr_t>(smem_raw) + 1023) &
                                                       ~std::uintptr_t(1023));
  // Output staging per epilogue warp: 32 x 32 complex64 (2 KB when DEEP).
  float2* staging = reinterpret_cast<float2*>(smem + STAGE_REGION);
  std::uint64_t* full = reinterpret_cast<std::uint64_t*>(smem + STAGE_REGION + STG_BYTES);
  std::uint64_t* empty = full + NST;
  std::uint64_t* acc_full = empty + NST;       // [NBUF]: a chunk accumulator is complete
  std::uint64_t* acc_empty = acc_full + NBUF;  // [NBUF]: a chunk accumulator was drained
  std::uint64_t* mma_done = acc_empty + NBUF;  // every issued MMA has completed
  std::uint32_t* tmem_slot = reinterpret_cast<std::uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // Work items (tiles) of this CTA (of this pair): first, first + stride, ...
  const std::uint32_t rank = PAIR ? cluster_rank() : 0;
  const int first = PAIR ? blockIdx.x / 2 : blockIdx.x;
  const int stride = PAIR ? gridDim.x / 2 : gridDim.x;
  const int tiles_m = (m + TM - 1) / TM;
  const int tiles_n = (n + TBN - 1) / TBN;
  const int per_batch = tiles_m * tiles_n;
  const int total = per_batch * batches;
  // Tiles run in groups of 8 row-tiles so that the CTAs working at one time
  // share A rows and B columns in L2.
  auto tile_of = [&](int t, int& m0, int& n0, int& batch) {
    batch = t / per_batch;
    const int r = t % per_batch;
    const int per_group = 8 * tiles_n;
    const int group = r / per_group, in_group = r % per_group;
    const int group_m = min(8, tiles_m - group * 8);
    m0 = (group * 8 + in_group % group_m) * TM + int(rank) * BM;
    n0 = (in_group / group_m) * TBN;
  };
  // Waits on barriers that the other CTA of a pair (or its MMA commits) may
  // complete use cluster scope.
  auto wait = [&](std::uint64_t* bar, std::uint32_t parity, int code) {
    return PAIR ? mbar_wait_cluster(bar, parity, abort_flag, err, code) : mbar_wait(bar, parity, abort_flag, err, code);
  };
  auto commit = [&](std::uint64_t* bar) {
    if constexpr (PAIR)
      umma_commit_pair(bar);
    else
      umma_commit(bar);
  };
  const int kblocks = (k + KSTEP - 1) / KSTEP;
  const int chunks = (kblocks + CHUNK - 1) / CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NBUF; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], PAIR ? 2 * EPI : EPI);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(TMEM_COLS));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(TMEM_COLS));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if constexpr (PAIR) cluster_sync();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const std::uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // Producer: stage s (phase ph) of the CTA-wide k-step count g.
    int g = 0, s = 0;
    std::uint32_t ph = 0;
    for (int t = first; t < total && !*abort_flag; t += stride) {
      int m0, n0, batch;
      tile_of(t, m0, n0, batch);
      for (int kb = 0; kb < kblocks; ++kb) {
        if (g >= NST && !wait(&empty[s], ph ^ 1u, 1)) break;
        std::uint8_t* st = smem + s * SBYTES;
        if constexpr (PAIR) {
          // This CTA's A rows (re, im) and its half of the B operands: CTA 0
          // Br (x = 0) and -Bi (64), CTA 1 Bi (32) and Br (0).
          if (rank == 0) mbar_expect_tx(&full[s], 2 * SBYTES);
          const std::uint32_t bar = peer_addr(&full[s], 0);
          tma_load_4d_pair(map_a, bar, st, 0, m0, kb, batch);
          tma_load_4d_pair(map_a, bar, st + F16_BLOCK, 32, m0, kb, batch);
          tma_load_4d_pair(map_b, bar, st + 2 * F16_BLOCK, rank ? 32 : 0, n0, kb, batch);
          tma_load_4d_pair(map_b, bar, st + 3 * F16_BLOCK, rank ? 0 : 64, n0, kb, batch);
        } else {
          mbar_expect_tx(&full[s], SBYTES);
          if constexpr (KIND == KIND_FP16) {
            // A: one box of whole 128-byte rows (16 KB); B: planes x = 64
            // (-im), 0 (re) and 32 (im), hi and lo each.
            tma_load_4d(map_a, &full[s], st, 0, m0, kb, batch);
            tma_load_4d(map_b, &full[s], st + 2 * F16_BLOCK, 64, n0, kb, batch);
            tma_load_4d(map_b, &full[s], st + 2 * F16_BLOCK + F16_BBLOCK, 0, n0, kb, batch);
            tma_load_4d(map_b, &full[s], st + 2 * F16_BLOCK + 2 * F16_BBLOCK, 32, n0, kb, batch);
          } else {
            tma_load_4d(map_a, &full[s], st, 0, m0, kb, batch);
            tma_load_4d(map_b, &full[s], st + TILE_A, 0, n0, kb, batch);
          }
          if constexpr (KIND == KIND_BF16) {
            tma_load_4d(map_a2, &full[s], st + 2 * TILE_A, 0, m0, kb, batch);
            tma_load_4d(map_b2, &full[s], st + 2 * TILE_A + TAIL, 0, n0, kb, batch);
          }
        }
        ++g;
        if (++s == NST) {
          s = 0;
          ph ^= 1u;
        }
      }
    }
    if (*abort_flag && rank == 0) {
      // Let the copies already issued land before the CTA's shared memory
      // is released (bounded as well; a pair's copies complete on CTA 0).
      for (int q = g > NST ? g - NST : 0; q < g; ++q) {
        const unsigned long long t0 = now_ns();
        while (!mbar_test(&full[q % NST], (q / NST) & 1) && now_ns() - t0 < WAIT_NS) {
        }
      }
    }
  } else if (warp == 1 && lane == 0 && rank == 0) {
    // MMA issuer (of the pair: CTA 0). Planes in a stage: A re_hi, re_lo,
    // im_hi, im_lo, then B.
    // Chunk c (CHUNK k-steps of one tile; c counts across tiles) accumulates
    // from zero into TMEM buffer c % 2; the epilogue warps add it into their
    // FP32 registers and free it.
    const std::uint32_t idp = idesc_kind<KIND>(BM, TBN, false), idn = idesc_kind<KIND>(BM, TBN, true);
    // 3xFP16: descriptor of stage 0's A re hi plane; the stage's others
    // follow at fixed offsets (umma_f16_kstep), stage s at + s SBYTES / 16.
    const std::uint64_t f16d0 = smem_desc_sw128(smem_u32(smem));
    const std::uint32_t f16_hia = std::uint32_t(f16d0 >> 32);
    const std::uint32_t f16_hib = std::uint32_t(smem_desc_sw64(smem_u32(smem)) >> 32);
    std::uint32_t f16_lo = std::uint32_t(f16d0);
    // Stage s with phase bit ph, k-step kc of chunk c: counters, not
    // divisions, since this thread's instruction stream paces the MMAs.
    int s = 0, c = 0, kc = 0;
    std::uint32_t ph = 0;
    bool go = true;
    for (int t = first; t < total && go; t += stride) {
      kc = 0;
      for (int kb = 0; kb < kblocks; ++kb) {
        const int buf = c % NBUF;
        const bool first = kc == 0;
        if (first && c >= NBUF) {
          // The epilogue's TMEM reads of this buffer precede the MMAs that
          // overwrite it.
          if (!wait(&acc_empty[buf], ((c / NBUF) - 1) & 1, 4)) {
            go = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
        }
        // Operand stages need no fence: the TMA's complete_tx on the barrier
        // orders its shared-memory writes before the MMAs' reads.
        if (!wait(&full[s], ph, 2)) {
          go = false;
          break;
        }
        const std::uint32_t d_re = tmem + buf * 2 * TBN, d_im = d_re + TBN;
        const std::uint32_t a0 = smem_u32(smem + s * SBYTES);
        const std::uint32_t acc = first ? 0u : 1u;
        if constexpr (PAIR) {
          // M = 256 over the pair; B rows (Br; Bi) at the stage's B offset
          // and (-Bi; Br) 8 KB further, each half in its own CTA.
          const std::uint32_t idw = idesc_f16(2 * BM, 2 * BN, false);
          const std::uint32_t ar = a0, ai = a0 + F16_BLOCK, b1 = a0 + 2 * F16_BLOCK, b2 = a0 + 3 * F16_BLOCK;
          const std::uint64_t arh = smem_desc_sw64(ar), arl = smem_desc_sw64(ar + 32);
          const std::uint64_t aih = smem_desc_sw64(ai), ail = smem_desc_sw64(ai + 32);
          const std::uint64_t b1h = smem_desc_sw64(b1), b1l = smem_desc_sw64(b1 + 32);
          const std::uint64_t b2h = smem_desc_sw64(b2), b2l = smem_desc_sw64(b2 + 32);
          umma_f16_pair(d_re, arh, b1l, idw, acc);
          umma_f16_pair(d_re, arl, b1h, idw, 1);
          umma_f16_pair(d_re, aih, b2l, idw, 1);
          umma_f16_pair(d_re, ail, b2h, idw, 1);
          umma_f16_pair(d_re, arh, b1h, idw, 1);
          umma_f16_pair(d_re, aih, b2h, idw, 1);
          (void)d_im;
        } else if constexpr (KIND == KIND_FP16) {
          // One M = 128, N = 256 product gives C_re (columns 0..127) and
          // C_im (128..255) together: Ar against the B rows (Br; Bi) and Ai
          // against (-Bi; Br), both read from the stage's B blocks
          // (-Bi, Br, Bi). Six MMAs per k-step, small terms first.
          // Stage s's descriptors: stage 0's with the start address moved
          // by s * SBYTES (the 14-bit field cannot carry: shared memory is
          // below 256 KB).
          umma_f16_kstep(d_re, f16_lo, f16_hia, f16_hib, idesc_f16(BM, 2 * TBN, false), acc, F16_BBLOCK / 16);
          (void)d_im;
        } else {
          const std::uint32_t b0 = a0 + TILE_A;
          const std::uint64_t arh = smem_desc_sw128(a0), arl = smem_desc_sw128(a0 + 32),
                              aih = smem_desc_sw128(a0 + 64), ail = smem_desc_sw128(a0 + 96);
          const std::uint64_t brh = smem_desc_sw128(b0), brl = smem_desc_sw128(b0 + 32),
                              bih = smem_desc_sw128(b0 + 64), bil = smem_desc_sw128(b0 + 96);
          if constexpr (KIND == KIND_BF16) {
            // Pieces 0 and 1 sit in the 128-byte rows (re0 re1 im0 im1, named
            // *h and *l above), piece 2 in the 64-byte rows (re2 im2). Per real
            // product x*y the terms x2y0, x1y1, x0y2 (~2^-16), x1y0, x0y1
            // (~2^-8) and x0y0, smallest first.
            const std::uint32_t at = a0 + 2 * TILE_A, bt = at + TAIL;
            const std::uint64_t ar2 = smem_desc_sw64(at), ai2 = smem_desc_sw64(at + 32);
            const std::uint64_t br2 = smem_desc_sw64(bt), bi2 = smem_desc_sw64(bt + 32);
            // C_re = Ar Br - Ai Bi
            umma<KIND>(d_re, ar2, brh, idp, acc);
            umma<KIND>(d_re, arl, brl, idp, 1);
            umma<KIND>(d_re, arh, br2, idp, 1);
            umma<KIND>(d_re, ai2, bih, idn, 1);
            umma<KIND>(d_re, ail, bil, idn, 1);
            umma<KIND>(d_re, aih, bi2, idn, 1);
            umma<KIND>(d_re, arl, brh, idp, 1);
            umma<KIND>(d_re, arh, brl, idp, 1);
            umma<KIND>(d_re, ail, bih, idn, 1);
            umma<KIND>(d_re, aih, bil, idn, 1);
            umma<KIND>(d_re, arh, brh, idp, 1);
            umma<KIND>(d_re, aih, bih, idn, 1);
            // C_im = Ar Bi + Ai Br
            umma<KIND>(d_im, ar2, bih, idp, acc);
            umma<KIND>(d_im, arl, bil, idp, 1);
            umma<KIND>(d_im, arh, bi2, idp, 1);
            umma<KIND>(d_im, ai2, brh, idp, 1);
            umma<KIND>(d_im, ail, brl, idp, 1);
            umma<KIND>(d_im, aih, br2, idp, 1);
            umma<KIND>(d_im, arl, bih, idp, 1);
            umma<KIND>(d_im, arh, bil, idp, 1);
            umma<KIND>(d_im, ail, brh, idp, 1);
            umma<KIND>(d_im, aih, brl, idp, 1);
            umma<KIND>(d_im, arh, bih, idp, 1);
            umma<KIND>(d_im, aih, brh, idp, 1);
          } else {
            // The small hi*lo terms go first and the two large hi*hi terms
            // last, so only those two additions round against a large
            // accumulator.
            umma<KIND>(d_re, arh, brl, idp, acc);
            umma<KIND>(d_re, arl, brh, idp, 1);
            umma<KIND>(d_re, aih, bil, idn, 1);
            umma<KIND>(d_re, ail, bih, idn, 1);
            umma<KIND>(d_re, arh, brh, idp, 1);
            umma<KIND>(d_re, aih, bih, idn, 1);
            umma<KIND>(d_im, arh, bil, idp, acc);
            umma<KIND>(d_im, arl, bih, idp, 1);
            umma<KIND>(d_im, aih, brl, idp, 1);
            umma<KIND>(d_im, ail, brh, idp, 1);
            umma<KIND>(d_im, arh, bih, idp, 1);
            umma<KIND>(d_im, aih, brh, idp, 1);
          }
        }
        commit(&empty[s]);
        if (++kc == CHUNK || kb == kblocks - 1) {
          commit(&acc_full[buf]);
          ++c;
          kc = 0;
        }
        f16_lo += SBYTES >> 4;
        if (++s == NST) {
          s = 0;
          ph ^= 1;
          f16_lo -= NST * (SBYTES >> 4);
        }
      }
    }
    commit(mma_done);
  } else if (warp >= 2) {
    // Epilogue: warp w reads TMEM lanes [32 (w % 4), 32 (w % 4) + 32) and one
    // half of the tile's columns. The tensor core's FP32 accumulation rounds
    // toward zero; keeping each chunk short and adding the chunks here with
    // round-to-nearest keeps the product as accurate as FP32 arithmetic.
    const int q = warp % 4;
    const int part = (warp - 2) / 4;  // which COLS-wide share of the columns
    const int row = q * 32 + lane;
    float2* stg =
        reinterpret_cast<float2*>(reinterpret_cast<std::uint8_t*>(staging) + (warp - 2) * (STG_BYTES / EPI));
    int c = 0;
    bool ok = true;
    const float beta = debias_beta<KIND>(err, CHUNK, kblocks);
    // A pair's acc_empty barriers live in CTA 0.
    const std::uint32_t drained0 = PAIR ? peer_addr(&acc_empty[0], 0) : 0u;
    const std::uint32_t drained1 = PAIR ? peer_addr(&acc_empty[1], 0) : 0u;
    for (int t = first; t < total && ok; t += stride) {
      int m0, n0, batch;
      tile_of(t, m0, n0, batch);
      const int ncols = n - n0 - part * COLS;
      // 3xFP16 scale exponents of the tile's store: the row's (unless A's
      // blocks are applied per chunk) and, per 32-column piece, that of
      // column j0 + lane. Loaded before the chunks are drained, so that
      // their latency is hidden behind the drain.
      int ea = 0, eb0 = 0, eb1 = 0;
      bool fast = true;
      if (KIND == KIND_FP16) {
        ea = (a_blocks == 0 && m0 + row < m) ? exp_a[std::uint64_t(batch) * m + m0 + row] : 0;
        const int* eb = exp_b + std::uint64_t(batch) * n + n0 + part * COLS;
        eb0 = lane < ncols ? eb[lane] : 0;
        eb1 = COLS > 32 && 32 + lane < ncols ? eb[32 + lane] : eb0;
        // When every scale 2^-(ea + eb) of the warp's block is a normal
        // float, each element takes one multiply by it (exact unless the
        // result leaves the normal range, then rounded as ldexpf rounds).
        const int lo = __reduce_min_sync(0xffffffffu, ea) + __reduce_min_sync(0xffffffffu, min(eb0, eb1));
        const int hi = __reduce_max_sync(0xffffffffu, ea) + __reduce_max_sync(0xffffffffu, max(eb0, eb1));
        fast = hi <= 126 && lo >= -127;
      }
      float tre[COLS], tim[COLS];
#pragma unroll
      for (int j = 0; j < COLS; ++j) tre[j] = tim[j] = 0.f;
      // A's block exponent of a chunk is fetched one chunk ahead, so its
      // load latency stays out of the drain.
      const bool blocked = KIND == KIND_FP16 && a_blocks > 0 && m0 + row < m;
      const int* eblk = blocked ? exp_a + (std::uint64_t(batch) * m + m0 + row) * a_blocks : nullptr;
      int e_next = blocked ? eblk[0] : 0;
      for (int cc = 0; cc < chunks; ++cc, ++c) {
        const int buf = c % NBUF;
        const int e_blk = e_next;
        if (blocked && cc + 1 < chunks) e_next = eblk[((cc + 1) * CHUNK * KSTEP) / 32];
        if (!wait(&acc_full[buf], (c / NBUF) & 1, 3)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // Scale of this chunk: 1, or 2^-e of A's block for this row.
        const float sa = scale2(1.f, -e_blk);
        const std::uint32_t base = tmem + (std::uint32_t(q * 32) << 16) + buf * 2 * TBN + part * COLS;
#pragma unroll
        for (int j0 = 0; j0 < COLS; j0 += 16) {
          // 16 columns of re and of im per round trip: with the 128 running
          // sums that keeps the epilogue within its 168 registers.
          std::uint32_t vr[16], vi[16];
          TMEM_LD16(base + j0, vr);
          TMEM_LD16(base + TBN + j0, vi);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            tre[j0 + j] = fmaf(__uint_as_float(vr[j]), sa, tre[j0 + j]);
            tim[j0 + j] = fmaf(__uint_as_float(vi[j]), sa, tim[j0 + j]);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) {
          if constexpr (PAIR)
            mbar_arrive_remote(buf ? drained1 : drained0);
          else
            mbar_arrive(&acc_empty[buf]);
        }
      }
      if (!ok) break;
      // The MMA issuer already works on the next tile. The warp's 32 x 64
      // block leaves in two 32 x 32 pieces through its staging area.
      // Output element (re, im) of column j of the piece: scaled by
      // 2^-(ea + eb_j), eb_j held by lane j. Otherwise by two powers of two
      // 2^e1 2^e2 (e1 + e2 = e, each clamped to the normal range): the first
      // multiply is exact whenever the result is normal, and an exponent
      // beyond +-252 only arises for results far outside the float range.
      auto out = [&](float re, float im, int ebl, int j) -> float2 {
        re = fmaf(re, beta, re);
        im = fmaf(im, beta, im);
        if (KIND != KIND_FP16) return make_float2(re, im);
        const int ebj = __shfl_sync(0xffffffffu, ebl, j);
        if (fast) {
          const float sc = __uint_as_float(std::uint32_t(127 - ea - ebj) << 23);
          return make_float2(re * sc, im * sc);
        }
        const int e = -(ea + ebj), e1 = min(max(e >> 1, -126), 127), e2 = min(max(e - e1, -126), 127);
        const float s1 = __uint_as_float(std::uint32_t(e1 + 127) << 23);
        const float s2 = __uint_as_float(std::uint32_t(e2 + 127) << 23);
        return make_float2(re * s1 * s2, im * s1 * s2);
      };
      float2* cb = C + std::uint64_t(batch) * c_batch_stride;
#pragma unroll
      for (int j0 = 0; j0 < COLS; j0 += 32) {
        const int ebl = j0 ? eb1 : eb0;
        if constexpr (DEEP) {
          // Four boxes of 32 rows x 8 complex per piece, 64-byte swizzle
          // (16-byte unit u of row r at r * 64 + ((u ^ (r / 2) % 4) * 16)).
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            if (lane == 0) bulk_wait_read();
            __syncwarp();
#pragma unroll
            for (int jj = 0; jj < 8; jj += 2) {
              const int j = 8 * b + jj;
              const float2 v0 = out(tre[j0 + j], tim[j0 + j], ebl, j);
              const float2 v1 = out(tre[j0 + j + 1], tim[j0 + j + 1], ebl, j + 1);
              const int u = jj / 2;
              float4* dst = reinterpret_cast<float4*>(reinterpret_cast<std::uint8_t*>(stg) + lane * 64 +
                                                      ((u ^ ((lane >> 1) & 3)) << 4));
              *dst = make_float4(v0.x, v0.y, v1.x, v1.y);
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
              const int x = 2 * (n0 + part * COLS + j0 + 8 * b), y = m0 + q * 32;
              if (y < m && x < 2 * n) tma_store_3d(map_c, stg, x, y, batch);
              bulk_commit();
            }
          }
        } else if (tma_c || EPI != EPI_WARPS) {  // the wide kernel always stores by TMA
          // Boxes of 32 rows x 16 complex in the 128-byte swizzle (16-byte
          // unit u of row r at r * 128 + ((u ^ r % 8) * 16)), stored by TMA
          // from two 4 KB slots in turn; a slot is rewritten once the box
          // stored from it two boxes earlier was read (one commit group per
          // box, at most one other still reading).
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            // Two slots: a box waits for the one stored two boxes earlier;
            // one slot: for the previous box.
            std::uint8_t* slot = reinterpret_cast<std::uint8_t*>(stg) + (b % SLOTS) * 4096;
            if (lane == 0) {
              if constexpr (SLOTS >= 2)
                bulk_wait_read1();
              else
                bulk_wait_read();
            }
            __syncwarp();
#pragma unroll
            for (int jj = 0; jj < 16; jj += 2) {
              const int j = 16 * b + jj;
              const float2 v0 = out(tre[j0 + j], tim[j0 + j], ebl, j);
              const float2 v1 = out(tre[j0 + j + 1], tim[j0 + j + 1], ebl, j + 1);
              const int u = jj / 2;
              float4* dst = reinterpret_cast<float4*>(slot + lane * 128 + ((u ^ (lane & 7)) << 4));
              *dst = make_float4(v0.x, v0.y, v1.x, v1.y);
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
              const int x = 2 * (n0 + part * COLS + j0 + 16 * b), y = m0 + q * 32;
              if (y < m && x < 2 * n) tma_store_3d(map_c, slot, x, y, batch);
              bulk_commit();
            }
          }
        } else {
          // Element (r, j) of the piece sits at r * 32 + (j ^ r); the warp
          // stores whole 32-column row pieces.
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            stg[lane * 32 + (j ^ lane)] = out(tre[j0 + j], tim[j0 + j], ebl, j);
          }
          __syncwarp();
          for (int r = 0; r < 32; ++r) {
            const int gr = m0 + q * 32 + r;
            if (gr < m && j0 + lane < ncols)
              cb[std::uint64_t(gr) * n + n0 + part * COLS + j0 + lane] = stg[r * 32 + (lane ^ r)];
          }
          __syncwarp();
        }
      }
    }
    // Every bulk store has written global memory before the CTA ends.
    if (tma_c && lane == 0) bulk_wait_all();
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    // Release TMEM only after every MMA this CTA issued (or, in a pair, that
    // read this CTA's shared memory) has completed; the wait is immediate
    // unless the pipeline was abandoned.
    const unsigned long long t0 = now_ns();
    while (!(PAIR ? mbar_test_cluster(mma_done, 0) : mbar_test(mma_done, 0)) && now_ns() - t0 < WAIT_NS) {
    }
  }
  if constexpr (PAIR) {
    __syncthreads();
    cluster_sync();
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

__global__ void __launch_bounds__(THREADS, 1)
    cgemm_tf32x3_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                        const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m, int n,
                        int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err, int CHUNK) {
  cgemm_split_body<KIND_TF32>(&map_a, &map_b, nullptr, nullptr, &map_c, tma_c != 0, C, m, n, k, batches, c_batch_stride, err, CHUNK,
                              nullptr, nullptr, 0);
}

__global__ void __launch_bounds__(THREADS, 1)
    cgemm_fp16x3_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                        const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m, int n,
                        int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err, int CHUNK,
                        const int* __restrict__ exp_a, const int* __restrict__ exp_b, int a_blocks) {
  cgemm_split_body<KIND_FP16>(&map_a, &map_b, nullptr, nullptr, &map_c, tma_c != 0, C, m, n, k, batches, c_batch_stride, err, CHUNK,
                              exp_a, exp_b, a_blocks);
}

// The 3xFP16 product with five stages (see cgemm_split_body).
__global__ void __launch_bounds__(THREADS, 1)
    cgemm_fp16x3_deep_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                             const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m,
                             int n, int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err,
                             int CHUNK, const int* __restrict__ exp_a, const int* __restrict__ exp_b, int a_blocks) {
  cgemm_split_body<KIND_FP16, false, true>(&map_a, &map_b, nullptr, nullptr, &map_c, tma_c != 0, C, m, n, k, batches,
                                           c_batch_stride, err, CHUNK, exp_a, exp_b, a_blocks);
}

// The 3xFP16 product on CTA pairs (see cgemm_split_body).
__global__ void __launch_bounds__(WIDE_THREADS, 1)
    cgemm_fp16x3_wide_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                             const __grid_constant__ CUtensorMap map_c, float2* __restrict__ C, int m, int n, int k,
                             int batches, std::uint64_t c_batch_stride, int* __restrict__ err, int CHUNK,
                             const int* __restrict__ exp_a, const int* __restrict__ exp_b, int a_blocks) {
  cgemm_split_body<KIND_FP16, false, false, WIDE_EPI_WARPS>(&map_a, &map_b, nullptr, nullptr, &map_c, true, C, m,
                                                           n, k, batches, c_batch_stride, err, CHUNK, exp_a, exp_b,
                                                           a_blocks);
}

__global__ void __launch_bounds__(THREADS, 1)
    cgemm_fp16x3_narrow_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                               const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m,
                               int n, int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err,
                               int CHUNK, const int* __restrict__ exp_a, const int* __restrict__ exp_b, int a_blocks) {
  cgemm_split_body<KIND_FP16, false, false, EPI_WARPS, 64>(&map_a, &map_b, nullptr, nullptr, &map_c, tma_c != 0, C, m,
                                                          n, k, batches, c_batch_stride, err, CHUNK, exp_a, exp_b,
                                                          a_blocks);
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    cgemm_fp16x3_pair_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                             const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m,
                             int n, int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err,
                             int CHUNK, const int* __restrict__ exp_a, const int* __restrict__ exp_b, int a_blocks) {
  cgemm_split_body<KIND_FP16, true>(&map_a, &map_b, nullptr, nullptr, &map_c, tma_c != 0, C, m, n, k, batches,
                                    c_batch_stride, err, CHUNK, exp_a, exp_b, a_blocks);
}

__global__ void __launch_bounds__(THREADS, 1)
    cgemm_bf16x3_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                        const __grid_constant__ CUtensorMap map_a2, const __grid_constant__ CUtensorMap map_b2,
                        const __grid_constant__ CUtensorMap map_c, int tma_c, float2* __restrict__ C, int m, int n,
                        int k, int batches, std::uint64_t c_batch_stride, int* __restrict__ err, int CHUNK) {
  cgemm_split_body<KIND_BF16>(&map_a, &map_b, &map_a2, &map_b2, &map_c, tma_c != 0, C, m, n, k, batches, c_batch_stride, err, CHUNK,
                              nullptr, nullptr, 0);
}

// ---- CTA-pair kernel (cta_group::2) -------------------------------------------
//
// Same arithmetic as above on a 256 x 128 output tile shared by the two CTAs
// of a cluster: CTA r holds A rows m0 + 128 r .. + 127 and B rows (output
// columns) n0 + 64 r .. + 63 in its shared memory, and one MMA of M = 256,
// N = 128 issued by the even CTA reads both CTAs' tiles and writes each
// CTA's 128 rows into that CTA's TMEM. Per k-step an SM now reads 6 KB of
// operands per MMA (its A rows and half of B) instead of 8 KB, and TMA
// writes 24 KB instead of 32 KB. Measured slower than the single-CTA tile
// on the products of the 7x7 plan; opt-in per shape.
//
// Synchronisation across the pair:
//   * both CTAs' TMA loads complete on the even CTA's full[s] barrier, which
//     expects the bytes of both;
//   * MMA commits are multicast to both CTAs (empty[s], acc_full[b],
//     mma_done), so each CTA's producer and epilogue wait on local barriers;
//   * both CTAs' epilogue warps arrive on the even CTA's acc_empty[b];
//   * cluster barriers after set-up (barriers initialised, TMEM allocated)
//     and before TMEM is released.
constexpr int PBM = 128;          // rows per CTA (256 per pair)
constexpr int PBN = 128;          // output columns per pair
constexpr int PBN_CTA = PBN / 2;  // B rows per CTA
constexpr int P_STAGES = 8;
constexpr int P_TILE_A = PBM * 128;
constexpr int P_TILE_B = PBN_CTA * 128;
constexpr int P_STAGE_BYTES = P_TILE_A + P_TILE_B;
constexpr int P_SMEM_BYTES = P_STAGES * P_STAGE_BYTES + 1024 + 256;
constexpr int P_GROUP = 4;  // pair-row tiles per raster group

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    cgemm_tf32x3_pair_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                             float2* __restrict__ C, int m, int n, int k, std::uint64_t c_batch_stride,
                             int* __restrict__ err, int CHUNK) {
  extern __shared__ __align__(1024) std::uint8_t smem_raw[];
  std::uint8_t* smem = reinterpret_cast<std::uint8_t*>((reinterpret_cast<std::uintptr_t>(smem_raw) + 1023) &
                                                       ~std::uintptr_t(1023));
  std::uint64_t* full = reinterpret_cast<std::uint64_t*>(smem + P_STAGES * P_STAGE_BYTES);
  std::uint64_t* empty = full + P_STAGES;
  std::uint64_t* acc_full = empty + P_STAGES;
  std::uint64_t* acc_empty = acc_full + 2;  // used in the even CTA only
  std::uint64_t* mma_done = acc_empty + 2;
  std::uint32_t* tmem_slot = reinterpret_cast<std::uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const std::uint32_t rank = cluster_rank();
  const int pair = blockIdx.x / 2;
  const int tiles_m = (m + 2 * PBM - 1) / (2 * PBM);
  const int tiles_n = (n + PBN - 1) / PBN;
  const int per_group = P_GROUP * tiles_n;
  const int group = pair / per_group, in_group = pair % per_group;
  const int group_m = min(P_GROUP, tiles_m - group * P_GROUP);
  const int m0 = (group * P_GROUP + in_group % group_m) * (2 * PBM) + int(rank) * PBM;
  const int n0 = (in_group / group_m) * PBN;
  const int batch = blockIdx.z;
  const int kblocks = (k + BK - 1) / BK;
  const int chunks = (kblocks + CHUNK - 1) / CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < P_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 2 * EPI_WARPS);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  cluster_sync();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const std::uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // Producer (both CTAs): this CTA's A rows and B rows, completing on the
    // even CTA's full barrier.
    int issued = 0;
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % P_STAGES;
      if (kb >= P_STAGES && !mbar_wait_cluster(&empty[s], ((kb / P_STAGES) - 1) & 1, abort_flag, err, 11)) break;
      std::uint8_t* st = smem + s * P_STAGE_BYTES;
      if (rank == 0) mbar_expect_tx(&full[s], 2 * P_STAGE_BYTES);
      const std::uint32_t bar = peer_addr(&full[s], 0);
      tma_load_4d_pair(&map_a, bar, st, 0, m0, kb, batch);
      tma_load_4d_pair(&map_b, bar, st + P_TILE_A, 0, n0 + int(rank) * PBN_CTA, kb, batch);
      issued = kb + 1;
    }
    if (*abort_flag && rank == 0) {
      for (int kb = issued > P_STAGES ? issued - P_STAGES : 0; kb < issued; ++kb) {
        const unsigned long long t0 = now_ns();
        while (!mbar_test_cluster(&full[kb % P_STAGES], (kb / P_STAGES) & 1) && now_ns() - t0 < WAIT_NS) {
        }
      }
    }
  } else if (warp == 1 && lane == 0 && rank == 0) {
    // MMA issuer of the pair (even CTA).
    const std::uint32_t idp = idesc_tf32(2 * PBM, PBN, false), idn = idesc_tf32(2 * PBM, PBN, true);
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % P_STAGES;
      const int c = kb / CHUNK, buf = c & 1;
      const bool first = kb % CHUNK == 0;
      if (first && c >= 2) {
        if (!mbar_wait_cluster(&acc_empty[buf], ((c >> 1) - 1) & 1, abort_flag, err, 14)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
      }
      if (!mbar_wait_cluster(&full[s], (kb / P_STAGES) & 1, abort_flag, err, 12)) break;
      const std::uint32_t d_re = tmem + buf * 2 * PBN, d_im = d_re + PBN;
      const std::uint32_t a0 = smem_u32(smem + s * P_STAGE_BYTES);
      const std::uint32_t b0 = a0 + P_TILE_A;
      const std::uint64_t arh = smem_desc_sw128(a0), arl = smem_desc_sw128(a0 + 32),
                          aih = smem_desc_sw128(a0 + 64), ail = smem_desc_sw128(a0 + 96);
      const std::uint64_t brh = smem_desc_sw128(b0), brl = smem_desc_sw128(b0 + 32),
                          bih = smem_desc_sw128(b0 + 64), bil = smem_desc_sw128(b0 + 96);
      const std::uint32_t acc = first ? 0u : 1u;
      umma_tf32_pair(d_re, arh, brl, idp, acc);
      umma_tf32_pair(d_re, arl, brh, idp, 1);
      umma_tf32_pair(d_re, aih, bil, idn, 1);
      umma_tf32_pair(d_re, ail, bih, idn, 1);
      umma_tf32_pair(d_re, arh, brh, idp, 1);
      umma_tf32_pair(d_re, aih, bih, idn, 1);
      umma_tf32_pair(d_im, arh, bil, idp, acc);
      umma_tf32_pair(d_im, arl, bih, idp, 1);
      umma_tf32_pair(d_im, aih, brl, idp, 1);
      umma_tf32_pair(d_im, ail, brh, idp, 1);
      umma_tf32_pair(d_im, arh, bih, idp, 1);
      umma_tf32_pair(d_im, aih, brh, idp, 1);
      umma_commit_pair(&empty[s]);
      if (kb % CHUNK == CHUNK - 1 || kb == kblocks - 1) umma_commit_pair(&acc_full[buf]);
    }
    umma_commit_pair(mma_done);
  } else if (warp >= 2) {
    // Epilogue (both CTAs): this CTA's 128 rows from its own TMEM.
    const int q = warp % 4;
    const int half = (warp - 2) / 4;
    const int row = q * 32 + lane;
    const std::uint32_t empty0 = peer_addr(&acc_empty[0], 0), empty1 = peer_addr(&acc_empty[1], 0);
    float tre[PBN / 2], tim[PBN / 2];
#pragma unroll
    for (int j = 0; j < PBN / 2; ++j) tre[j] = tim[j] = 0.f;
    bool ok = true;
    for (int c = 0; c < chunks; ++c) {
      const int buf = c & 1;
      if (!mbar_wait_cluster(&acc_full[buf], (c >> 1) & 1, abort_flag, err, 13)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const std::uint32_t base = tmem + (std::uint32_t(q * 32) << 16) + buf * 2 * PBN + half * (PBN / 2);
#pragma unroll
      for (int j0 = 0; j0 < PBN / 2; j0 += 32) {
        std::uint32_t vr[32], vi[32];
        TMEM_LD32(base + j0, vr);
        TMEM_LD32(base + PBN + j0, vi);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          tre[j0 + j] += __uint_as_float(vr[j]);
          tim[j0 + j] += __uint_as_float(vi[j]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive_remote(buf ? empty1 : empty0);
    }
    if (ok && m0 + row < m) {
      float2* crow =
          C + std::uint64_t(batch) * c_batch_stride + std::uint64_t(m0 + row) * n + n0 + half * (PBN / 2);
      const int ncols = n - n0 - half * (PBN / 2);
#pragma unroll
      for (int j = 0; j < PBN / 2; ++j)
        if (j < ncols) crow[j] = make_float2(tre[j], tim[j]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) {
    // Every MMA of the pair has completed before either CTA frees TMEM or
    // leaves (the MMAs read both CTAs' shared memory).
    const unsigned long long t0 = now_ns();
    while (!mbar_test_cluster(mma_done, 0) && now_ns() - t0 < WAIT_NS) {
    }
  }
  __syncthreads();
  cluster_sync();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// Splits complex64 rows into the four TF32 planes (round-to-nearest).
__device__ __forceinline__ float tf32_rn(float x) {
  std::uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Row access shared by the split kernels: one warp per row, lanes over k.
// A row whose start is 16-byte aligned (and k even) is read as float4 pairs.
struct RowReader {
  const float2* r;
  std::uint64_t k;
  bool vec;
  __device__ RowReader(const float2* row, std::uint64_t k_)
      : r(row), k(k_), vec(((reinterpret_cast<std::uintptr_t>(row) & 15) == 0) && (k_ % 2 == 0)) {}
  // Values kk and kk + 1 (kk even), zero beyond k.
  __device__ __forceinline__ void pair(std::uint64_t kk, float2& v0, float2& v1) const {
    if (kk >= k) {
      v0 = v1 = make_float2(0.f, 0.f);
    } else if (vec) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(r + kk));
      v0 = make_float2(v.x, v.y);
      v1 = make_float2(v.z, v.w);
    } else {
      v0 = r[kk];
      v1 = kk + 1 < k ? r[kk + 1] : make_float2(0.f, 0.f);
    }
  }
};

// Output layout per batch entry: [k / 8][row][plane][8] fp32 with planes
// re_hi, re_lo, im_hi, im_lo; k is padded to a multiple of 8 with zeros.
// k-step-major, so the 128 rows of one k-step that a tile loads are one
// contiguous 16 KB block. One warp per row; lane j covers k = 2j, 2j + 1 of
// every 64.
__global__ void __launch_bounds__(256) split_tf32_kernel(const float2* __restrict__ src, float* __restrict__ planes,
                                                         std::uint64_t rows, std::uint64_t k, std::uint64_t kpad,
                                                         std::uint64_t src_batch_stride) {
  const std::uint64_t b = blockIdx.y;
  const float2* sb = src + b * src_batch_stride;
  float* pb = planes + b * 4 * rows * kpad;
  const int lane = threadIdx.x % 32;
  const std::uint64_t warps = std::uint64_t(gridDim.x) * (blockDim.x / 32);
  for (std::uint64_t row = (std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; row < rows; row += warps) {
    const RowReader rd(sb + row * k, k);
#pragma unroll 4
    for (std::uint64_t kk = 2 * lane; kk < kpad; kk += 64) {
      float2 v0, v1;
      rd.pair(kk, v0, v1);
      const float rh0 = tf32_rn(v0.x), ih0 = tf32_rn(v0.y), rh1 = tf32_rn(v1.x), ih1 = tf32_rn(v1.y);
      float* o = pb + ((kk / 8) * rows + row) * 32 + (kk % 8);
      *reinterpret_cast<float2*>(o) = make_float2(rh0, rh1);
      *reinterpret_cast<float2*>(o + 8) = make_float2(tf32_rn(v0.x - rh0), tf32_rn(v1.x - rh1));
      *reinterpret_cast<float2*>(o + 16) = make_float2(ih0, ih1);
      *reinterpret_cast<float2*>(o + 24) = make_float2(tf32_rn(v0.y - ih0), tf32_rn(v1.y - ih1));
    }
  }
}

// 3xFP16 planes. One warp per row: the row's largest |re| or |im| sets a
// power-of-two scale e with max * 2^e in [2^14, 2^15) (FP16 holds up to
// 65504), then hi = fp16(x 2^e) and lo = fp16(x 2^e - hi) for re and im,
// both round-to-nearest, so x 2^e = hi + lo to ~22 significant bits.
// Output per batch entry: planes [k / 16][row][plane][16] fp16 (re_hi,
// re_lo, im_hi, im_lo, and with nplanes = 6 also -im_hi, -im_lo; one 128- or
// 192-byte row per k-step, k zero-padded to a multiple of 16) and the
// exponents [row] (int).
__global__ void __launch_bounds__(256) split_fp16_kernel(const float2* __restrict__ src, __half* __restrict__ planes,
                                                         int* __restrict__ exps, std::uint64_t rows, std::uint64_t k,
                                                         std::uint64_t kpad, std::uint64_t src_batch_stride,
                                                         int nplanes) {
  const std::uint64_t b = blockIdx.y;
  const float2* sb = src + b * src_batch_stride;
  __half* pb = planes + b * nplanes * rows * kpad;
  int* eb = exps + b * rows;
  const int lane = threadIdx.x % 32;
  const std::uint64_t warps = std::uint64_t(gridDim.x) * (blockDim.x / 32);
  for (std::uint64_t row = (std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; row < rows; row += warps) {
    const RowReader rd(sb + row * k, k);
    float mx = 0.f;
#pragma unroll 4
    for (std::uint64_t kk = 2 * lane; kk < k; kk += 64) {
      float2 v0, v1;
      rd.pair(kk, v0, v1);
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v0.x), fabsf(v0.y)), fmaxf(fabsf(v1.x), fabsf(v1.y))));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) {
      int ex;
      frexpf(mx, &ex);  // mx in [2^(ex-1), 2^ex)
      e = 15 - ex;
    }
    if (lane == 0) eb[row] = e;
#pragma unroll 4
    for (std::uint64_t kk = 2 * lane; kk < kpad; kk += 64) {
      float2 v0, v1;
      rd.pair(kk, v0, v1);
      const float r0 = ldexpf(v0.x, e), i0 = ldexpf(v0.y, e), r1 = ldexpf(v1.x, e), i1 = ldexpf(v1.y, e);
      const __half2 rh = __floats2half2_rn(r0, r1), ih = __floats2half2_rn(i0, i1);
      const float2 rhf = __half22float2(rh), ihf = __half22float2(ih);
      __half* o = pb + ((kk / 16) * rows + row) * (16 * nplanes) + (kk % 16);
      const __half2 il = __floats2half2_rn(i0 - ihf.x, i1 - ihf.y);
      *reinterpret_cast<__half2*>(o) = rh;
      *reinterpret_cast<__half2*>(o + 16) = __floats2half2_rn(r0 - rhf.x, r1 - rhf.y);
      *reinterpret_cast<__half2*>(o + 32) = ih;
      *reinterpret_cast<__half2*>(o + 48) = il;
      if (nplanes == 6) {
        *reinterpret_cast<__half2*>(o + 64) = __hneg2(ih);
        *reinterpret_cast<__half2*>(o + 80) = __hneg2(il);
      }
    }
  }
}

// BF16x3 planes: x = b0 + b1 + b2 with b0 = bf16(x), b1 = bf16(x - b0),
// b2 = bf16(x - b0 - b1), all round-to-nearest. Output per batch entry:
// main planes [k / 16][row][64] bf16 (re0, re1, im0, im1; 128 bytes per
// k-step) and tail planes [k / 16][row][32] bf16 (re2, im2; 64 bytes), k
// zero-padded to a multiple of 16.
__global__ void __launch_bounds__(256) split_bf16_kernel(const float2* __restrict__ src,
                                                         __nv_bfloat16* __restrict__ main_planes,
                                                         __nv_bfloat16* __restrict__ tail_planes, std::uint64_t rows,
                                                         std::uint64_t k, std::uint64_t kpad,
                                                         std::uint64_t src_batch_stride) {
  const std::uint64_t b = blockIdx.y;
  const float2* sb = src + b * src_batch_stride;
  __nv_bfloat16* mb = main_planes + b * 4 * rows * kpad;
  __nv_bfloat16* tb = tail_planes + b * 2 * rows * kpad;
  const int lane = threadIdx.x % 32;
  const std::uint64_t warps = std::uint64_t(gridDim.x) * (blockDim.x / 32);
  for (std::uint64_t row = (std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; row < rows; row += warps) {
    const RowReader rd(sb + row * k, k);
#pragma unroll 4
    for (std::uint64_t kk = 2 * lane; kk < kpad; kk += 64) {
      float2 v0, v1;
      rd.pair(kk, v0, v1);
      // Pieces of (re, im) of values kk and kk + 1, two at a time.
      const __nv_bfloat162 r0 = __floats2bfloat162_rn(v0.x, v1.x), i0 = __floats2bfloat162_rn(v0.y, v1.y);
      const float2 r0f = __bfloat1622float2(r0), i0f = __bfloat1622float2(i0);
      const float2 rr = make_float2(v0.x - r0f.x, v1.x - r0f.y), ir = make_float2(v0.y - i0f.x, v1.y - i0f.y);
      const __nv_bfloat162 r1 = __floats2bfloat162_rn(rr.x, rr.y), i1 = __floats2bfloat162_rn(ir.x, ir.y);
      const float2 r1f = __bfloat1622float2(r1), i1f = __bfloat1622float2(i1);
      const __nv_bfloat162 r2 = __floats2bfloat162_rn(rr.x - r1f.x, rr.y - r1f.y);
      const __nv_bfloat162 i2 = __floats2bfloat162_rn(ir.x - i1f.x, ir.y - i1f.y);
      const std::uint64_t slot = (kk / 16) * rows + row;
      __nv_bfloat16* m = mb + slot * 64 + (kk % 16);
      *reinterpret_cast<__nv_bfloat162*>(m) = r0;
      *reinterpret_cast<__nv_bfloat162*>(m + 16) = r1;
      *reinterpret_cast<__nv_bfloat162*>(m + 32) = i0;
      *reinterpret_cast<__nv_bfloat162*>(m + 48) = i1;
      __nv_bfloat16* t = tb + slot * 32 + (kk % 16);
      *reinterpret_cast<__nv_bfloat162*>(t) = r2;
      *reinterpret_cast<__nv_bfloat162*>(t + 16) = i2;
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) throw std::string("ERROR (qflex_gb300: tensor cores) --> cuTensorMapEncodeTiled unavailable");
  return fn;
}

// 4-D map over split planes laid out [batch][kpad / 8][rows][32] (fp32),
// box {32, box_rows, 1, 1} (one 128-byte row per tile row), 128-byte swizzle.
CUtensorMap plane_map(const float* base, std::uint64_t rows, std::uint64_t kpad, int batch, int box_rows) {
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  const std::uint64_t kb = kpad / 8;
  const cuuint64_t dims[4] = {32, rows, kb, (cuuint64_t)batch};
  const cuuint64_t strides[3] = {128, rows * 128, kb * rows * 128};
  const cuuint32_t box[4] = {32, (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides,
                           box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> cuTensorMapEncodeTiled failed: ") +
        std::to_string((int)r);
  return map;
}

// 4-D map over FP16 planes laid out [batch][kpad / 16][rows][row_halves]
// (64: re hi, lo, im hi, lo; 96: also -im hi, lo). Box {32, box_rows, 1, 1}:
// the hi and lo planes of one part as 64-byte rows, 64-byte swizzle, the
// part chosen by the box's x coordinate (0, 32, 64); or with box_inner = 64
// whole 128-byte rows (all four planes of A) in the 128-byte swizzle.
CUtensorMap plane_map_f16(const __half* base, std::uint64_t rows, std::uint64_t kpad, int batch, int box_rows,
                          int row_halves, int box_inner = 32) {
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  const std::uint64_t kb = kpad / 16, rb = std::uint64_t(row_halves) * 2;
  const cuuint64_t dims[4] = {(cuuint64_t)row_halves, rows, kb, (cuuint64_t)batch};
  const cuuint64_t strides[3] = {rb, rows * rb, kb * rows * rb};
  const cuuint32_t box[4] = {(cuuint32_t)box_inner, (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<__half*>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           box_inner == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> cuTensorMapEncodeTiled failed: ") +
        std::to_string((int)r);
  return map;
}

// 4-D map over BF16 planes laid out [batch][kpad / 16][rows][inner] with
// `inner` 64 (128-byte rows, 128-byte swizzle) or 32 (64-byte rows, 64-byte
// swizzle); box {inner, box_rows, 1, 1}.
CUtensorMap plane_map_bf16(const __nv_bfloat16* base, std::uint64_t rows, std::uint64_t kpad, int batch,
                           int box_rows, int inner) {
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  const std::uint64_t kb = kpad / 16, rb = std::uint64_t(inner) * 2;
  const cuuint64_t dims[4] = {(cuuint64_t)inner, rows, kb, (cuuint64_t)batch};
  const cuuint64_t strides[3] = {rb, rows * rb, kb * rows * rb};
  const cuuint32_t box[4] = {(cuuint32_t)inner, (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           inner == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> cuTensorMapEncodeTiled failed: ") +
        std::to_string((int)r);
  return map;
}

// 3-D map over C as floats [batch][m][2n] for the epilogue's bulk stores,
// box {32, 32, 1} (32 rows x 16 complex) in the 128-byte swizzle, or with
// `narrow` {16, 32, 1} (8 complex) in the 64-byte swizzle. False (and the
// epilogue stores with plain instructions) when C is not 16-byte aligned, n
// or the batch stride is odd, or QFLEX_TC_TMA_STORE=0.
bool output_map(float2* C, std::size_t m, std::size_t n, std::uint64_t batch_stride, int batch, CUtensorMap* map,
                bool narrow = false) {
  static const bool enabled = [] {
    const char* e = std::getenv("QFLEX_TC_TMA_STORE");
    return !(e && std::atoi(e) == 0);
  }();
  std::memset(map, 0, sizeof(*map));
  if (!enabled || (reinterpret_cast<std::uintptr_t>(C) & 15) || (n & 1) || (batch > 1 && (batch_stride & 1)))
    return false;
  const cuuint64_t dims[3] = {2 * n, m, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {n * 8, (batch > 1 ? batch_stride : m * n) * 8};
  const cuuint32_t box[3] = {narrow ? 16u : 32u, 32, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, C, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, narrow ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::string("ERROR (qflex_gb300: CUDA ") + what + ") --> " + cudaGetErrorString(e);
}

}  // namespace

bool tc_eligible(std::size_t m, std::size_t n, std::size_t k) {
  return m >= 64 && n >= 64 && k >= 16 && k % 4 == 0 && m < (1u << 31) && n < (1u << 31) && k < (1u << 31);
}

std::size_t tc_workspace_elems(std::size_t m, std::size_t n, std::size_t k) {
  // The largest of the 3xTF32 planes (4 fp32 per element), the 3xFP16
  // planes (4 fp16 per element of A, 6 of Bt) plus their exponents and the BF16x3
  // planes (6 bf16 per element, fewer than the 3xTF32 ones).
  const std::size_t tf32 = 4 * (m + n) * ((k + 7) / 8 * 8);
  const std::size_t fp16 = (2 * m + 3 * n) * ((k + 15) / 16 * 16) + (m + n) + m * ((k + 31) / 32) + 64;
  return tf32 > fp16 ? tf32 : fp16;
}

// Grid of the persistent single-CTA kernels: one CTA per SM (at most one
// per tile); QFLEX_TC_PERSIST=0 launches one CTA per tile instead.
unsigned persistent_grid(std::size_t tiles) {
  static const int sms = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
      v = 152;
    const char* e = std::getenv("QFLEX_TC_PERSIST");
    if (e && std::atoi(e) == 0) v = 0;
    return v;
  }();
  return (unsigned)(sms > 0 ? std::min<std::size_t>(tiles, (std::size_t)sms) : tiles);
}

TcConfig tc_default_config() {
  TcConfig c;
  // k-steps per TMEM chunk. The tensor core's FP32 accumulation truncates,
  // which shrinks every product by a fraction that grows with the chunk
  // (debias_beta). Measured on 256 amplitudes of the 16-slice 7x7 (1+32+1)
  // workload against the FP64 oracle (3xFP16): chunk 2 without compensation
  // shrinks every amplitude by 4.9e-6 (largest error 1.2e-5 of the RMS
  // amplitude), chunk 1 by 2.3e-6 (5.8e-6) at 7 % less throughput, chunk 2
  // with the compensation (the default) by 1e-7 (2.6e-6).
  if (const char* e = std::getenv("QFLEX_TC_CHUNK")) {
    const int v = std::atoi(e);
    if (v >= 1 && v <= 64) c.chunk = v;
  }
  // The single-CTA tile measured faster on every product of the 7x7
  // (1+32+1) plan; QFLEX_TC_PAIR=1 sends products with m >= 256 to the pair.
  if (const char* e = std::getenv("QFLEX_TC_PAIR"))
    if (std::atoi(e) == 1) c.variant = -1;
  if (const char* e = std::getenv("QFLEX_TC_DEEP"))
    if (std::atoi(e) == 1) c.variant = 2;
  return c;
}

void launch_cgemm_tf32x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t batch_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s) {
  if (!tc_eligible(m, n, k)) throw std::string("ERROR (qflex_gb300: tensor cores) --> shape not eligible");
  if (cfg.chunk < 1 || cfg.chunk > 64)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> chunk length must be 1..64");
  const int chunk = cfg.chunk;
  static std::once_flag attr;
  std::call_once(attr, [] {
    check(cudaFuncSetAttribute(cgemm_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
    check(cudaFuncSetAttribute(cgemm_tf32x3_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               P_SMEM_BYTES),
          "cudaFuncSetAttribute");
  });
  const bool use_pair = cfg.variant == 1 || (cfg.variant < 0 && m >= 2 * PBM);
  float* pa = workspace;
  const std::size_t kpad = (k + BK - 1) / BK * BK;
  float* pb = workspace + 4 * m * kpad * (std::size_t)batch;
  {
    dim3 ga((unsigned)std::min<std::uint64_t>((m + 7) / 8, 152 * 16), (unsigned)batch);
    split_tf32_kernel<<<ga, 256, 0, s>>>(A, pa, m, k, kpad, batch_stride);
    dim3 gb((unsigned)std::min<std::uint64_t>((n + 7) / 8, 152 * 16), (unsigned)batch);
    split_tf32_kernel<<<gb, 256, 0, s>>>(Bt, pb, n, k, kpad, bt_stride);
    check(cudaGetLastError(), "split_tf32");
  }
  if (use_pair) {
    const CUtensorMap ma = plane_map(pa, m, kpad, batch, PBM);
    const CUtensorMap mb = plane_map(pb, n, kpad, batch, PBN_CTA);
    const std::size_t pairs = ((m + 2 * PBM - 1) / (2 * PBM)) * ((n + PBN - 1) / PBN);
    dim3 grid((unsigned)(2 * pairs), 1, (unsigned)batch);
    cgemm_tf32x3_pair_kernel<<<grid, THREADS, P_SMEM_BYTES, s>>>(ma, mb, C, (int)m, (int)n, (int)k, batch_stride,
                                                                 err, chunk);
    check(cudaGetLastError(), "cgemm_tf32x3_pair");
    return;
  }
  const CUtensorMap ma = plane_map(pa, m, kpad, batch, BM);
  const CUtensorMap mb = plane_map(pb, n, kpad, batch, BN);
  const std::size_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  dim3 grid(persistent_grid(tiles * (std::size_t)batch), 1, 1);
  CUtensorMap mc;
  const int tma_c = output_map(C, m, n, batch_stride, batch, &mc) ? 1 : 0;
  cgemm_tf32x3_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(ma, mb, mc, tma_c, C, (int)m, (int)n, (int)k, batch,
                                                        batch_stride, err, chunk);
  check(cudaGetLastError(), "cgemm_tf32x3");
}

Fp16Workspace fp16_workspace(float* workspace, std::size_t m, std::size_t n, std::size_t k, int batch) {
  const std::size_t kpad = (k + 15) / 16 * 16, nb = (std::size_t)batch;
  Fp16Workspace w;
  __half* pa = reinterpret_cast<__half*>(workspace);
  __half* pb = pa + 4 * m * kpad * nb;
  w.a_planes = pa;
  w.b_planes = pb;
  w.a_exps = reinterpret_cast<int*>(pb + 6 * n * kpad * nb);
  w.b_exps = w.a_exps + m * nb;
  w.a_block_exps = w.b_exps + n * nb;
  return w;
}

void launch_cgemm_fp16x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t batch_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s, bool a_in_planes) {
  if (!tc_eligible(m, n, k)) throw std::string("ERROR (qflex_gb300: tensor cores) --> shape not eligible");
  if (cfg.chunk < 1 || cfg.chunk > 64)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> chunk length must be 1..64");
  if (a_in_planes && (k < 32 || (k & (k - 1)) != 0 || cfg.chunk > 2))
    throw std::string("ERROR (qflex_gb300: tensor cores) --> A in planes needs k = 2^j >= 32 and chunk <= 2");
  static std::once_flag attr;
  std::call_once(attr, [] {
    check(cudaFuncSetAttribute(cgemm_fp16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
    check(cudaFuncSetAttribute(cgemm_fp16x3_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
    check(cudaFuncSetAttribute(cgemm_fp16x3_deep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               DEEP_SMEM_BYTES),
          "cudaFuncSetAttribute");
    check(cudaFuncSetAttribute(cgemm_fp16x3_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
    check(cudaFuncSetAttribute(cgemm_fp16x3_narrow_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
  });
  const bool use_pair = cfg.variant == 1 || (cfg.variant < 0 && m >= 2 * BM);
  const std::size_t kpad = (k + 15) / 16 * 16;
  const Fp16Workspace w = fp16_workspace(workspace, m, n, k, batch);
  __half* pa = static_cast<__half*>(w.a_planes);
  __half* pb = static_cast<__half*>(w.b_planes);
  int* ea = a_in_planes ? w.a_block_exps : w.a_exps;
  int* eb = w.b_exps;
  {
    if (!a_in_planes) {
      dim3 ga((unsigned)std::min<std::uint64_t>((m + 7) / 8, 152 * 16), (unsigned)batch);
      split_fp16_kernel<<<ga, 256, 0, s>>>(A, pa, ea, m, k, kpad, batch_stride, 4);
    }
    dim3 gb((unsigned)std::min<std::uint64_t>((n + 7) / 8, 152 * 16), (unsigned)batch);
    split_fp16_kernel<<<gb, 256, 0, s>>>(Bt, pb, eb, n, k, kpad, bt_stride, 6);
    check(cudaGetLastError(), "split_fp16");
  }
  // A: whole 128-byte rows for the single-CTA kernels, re / im halves for
  // the pair; B: 64-byte halves.
  const CUtensorMap ma_rows = plane_map_f16(pa, m, kpad, batch, BM, 64, 64);
  const CUtensorMap ma = plane_map_f16(pa, m, kpad, batch, BM, 64);
  const CUtensorMap mb = plane_map_f16(pb, n, kpad, batch, BN, 96);
  CUtensorMap mc;
  const int tma_c = output_map(C, m, n, batch_stride, batch, &mc) ? 1 : 0;
  const int a_blocks = a_in_planes ? (int)(k / 32) : 0;
  if (use_pair) {
    // One cluster of two CTAs per pair of SMs, persistent over 256-row tiles.
    const std::size_t tiles = ((m + 2 * BM - 1) / (2 * BM)) * ((n + BN - 1) / BN) * (std::size_t)batch;
    // As many clusters as can be resident at once (SMs pair up within a
    // GPC), at most one per tile.
    static const int resident = [] {
      cudaLaunchConfig_t lc = {};
      lc.gridDim = dim3(2, 1, 1);
      lc.blockDim = dim3(THREADS, 1, 1);
      lc.dynamicSmemBytes = SMEM_BYTES;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 2;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      lc.attrs = at;
      lc.numAttrs = 1;
      int v = 0;
      if (cudaOccupancyMaxActiveClusters(&v, cgemm_fp16x3_pair_kernel, &lc) != cudaSuccess || v < 1) {
        cudaGetLastError();
        v = (int)persistent_grid(1u << 20) / 2;
      }
      return std::max(1, v);
    }();
    const unsigned clusters = (unsigned)std::min<std::size_t>(tiles, (std::size_t)resident);
    cgemm_fp16x3_pair_kernel<<<2 * clusters, THREADS, SMEM_BYTES, s>>>(
        ma, mb, mc, tma_c, C, (int)m, (int)n, (int)k, batch, batch_stride, err, cfg.chunk, ea, eb, a_blocks);
    check(cudaGetLastError(), "cgemm_fp16x3_pair");
    return;
  }
  const std::size_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  dim3 grid(persistent_grid(tiles * (std::size_t)batch), 1, 1);
  CUtensorMap mcn;
  if (cfg.variant == 2 && output_map(C, m, n, batch_stride, batch, &mcn, true)) {
    cgemm_fp16x3_deep_kernel<<<grid, THREADS, DEEP_SMEM_BYTES, s>>>(
        ma_rows, mb, mcn, 1, C, (int)m, (int)n, (int)k, batch, batch_stride, err, cfg.chunk, ea, eb, a_blocks);
    check(cudaGetLastError(), "cgemm_fp16x3_deep");
    return;
  }
  if (cfg.variant == 4) {
    // 64-column tiles: B boxes of 64 rows.
    const CUtensorMap mb64 = plane_map_f16(pb, n, kpad, batch, 64, 96);
    const std::size_t tiles64 = ((m + BM - 1) / BM) * ((n + 63) / 64);
    dim3 grid64(persistent_grid(tiles64 * (std::size_t)batch), 1, 1);
    cgemm_fp16x3_narrow_kernel<<<grid64, THREADS, SMEM_BYTES, s>>>(ma_rows, mb64, mc, tma_c, C, (int)m, (int)n, (int)k,
                                                                  batch, batch_stride, err, cfg.chunk, ea, eb, a_blocks);
    check(cudaGetLastError(), "cgemm_fp16x3_narrow");
    return;
  }
  if (cfg.variant == 3 && tma_c) {
    cgemm_fp16x3_wide_kernel<<<grid, WIDE_THREADS, SMEM_BYTES, s>>>(
        ma_rows, mb, mc, C, (int)m, (int)n, (int)k, batch, batch_stride, err, cfg.chunk, ea, eb, a_blocks);
    check(cudaGetLastError(), "cgemm_fp16x3_wide");
    return;
  }
  cgemm_fp16x3_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(ma_rows, mb, mc, tma_c, C, (int)m, (int)n, (int)k, batch,
                                                        batch_stride, err, cfg.chunk, ea, eb, a_blocks);
  check(cudaGetLastError(), "cgemm_fp16x3");
}

void launch_cgemm_bf16x3(const float2* A, const float2* Bt, float2* C, std::size_t m, std::size_t n,
                         std::size_t k, std::uint64_t batch_stride, std::uint64_t bt_stride, int batch,
                         float* workspace, int* err, const TcConfig& cfg, cudaStream_t s) {
  if (!tc_eligible(m, n, k)) throw std::string("ERROR (qflex_gb300: tensor cores) --> shape not eligible");
  if (cfg.chunk < 1 || cfg.chunk > 64)
    throw std::string("ERROR (qflex_gb300: tensor cores) --> chunk length must be 1..64");
  static std::once_flag attr;
  std::call_once(attr, [] {
    check(cudaFuncSetAttribute(cgemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES),
          "cudaFuncSetAttribute");
  });
  const std::size_t kpad = (k + 15) / 16 * 16;
  const std::size_t nb = (std::size_t)batch;
  __nv_bfloat16* am = reinterpret_cast<__nv_bfloat16*>(workspace);
  __nv_bfloat16* at = am + 4 * m * kpad * nb;
  __nv_bfloat16* bm = at + 2 * m * kpad * nb;
  __nv_bfloat16* bt = bm + 4 * n * kpad * nb;
  {
    dim3 ga((unsigned)std::min<std::uint64_t>((m + 7) / 8, 152 * 16), (unsigned)batch);
    split_bf16_kernel<<<ga, 256, 0, s>>>(A, am, at, m, k, kpad, batch_stride);
    dim3 gb((unsigned)std::min<std::uint64_t>((n + 7) / 8, 152 * 16), (unsigned)batch);
    split_bf16_kernel<<<gb, 256, 0, s>>>(Bt, bm, bt, n, k, kpad, bt_stride);
    check(cudaGetLastError(), "split_bf16");
  }
  const CUtensorMap ma = plane_map_bf16(am, m, kpad, batch, BM, 64);
  const CUtensorMap mb = plane_map_bf16(bm, n, kpad, batch, BN, 64);
  const CUtensorMap ma2 = plane_map_bf16(at, m, kpad, batch, BM, 32);
  const CUtensorMap mb2 = plane_map_bf16(bt, n, kpad, batch, BN, 32);
  const std::size_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  dim3 grid(persistent_grid(tiles * (std::size_t)batch), 1, 1);
  CUtensorMap mc;
  const int tma_c = output_map(C, m, n, batch_stride, batch, &mc) ? 1 : 0;
  cgemm_bf16x3_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(ma, mb, ma2, mb2, mc, tma_c, C, (int)m, (int)n, (int)k, batch,
                                                        batch_stride, err, cfg.chunk);
  check(cudaGetLastError(), "cgemm_bf16x3");
}

}  // namespace qfx

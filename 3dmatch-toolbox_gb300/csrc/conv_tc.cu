// tcgen05 implicit-GEMM 3D convolution (and plain GEMM) for sm_103a.
//
// Replaces cudnnConvolutionForward + cudnnAddTensor + in-place ReLU of Marvin
// (core/marvin.hpp:4639-4660, 5486) for conv2..conv7, conv8 and feat of
// core/3dmatch-net-test.json.
//
// Data layout ("chunk-planar"): an activation tensor of C channels over P
// positions is stored as C/8 chunks (BF16) or C/16 chunks (E4M3); chunk j is a
// contiguous [P][16 bytes] array.  Position p of an input grid of extent D is
// the linear index ((b*D + z)*D + y)*D + x.
//
// Convolution as GEMM over the *input* grid: output row p (valid when its
// x, y, z < D-2) is sum over taps (dz,dy,dx) of A[p + dz*D^2 + dy*D + dx] . W_tap.
// For one dz, the rows needed by all 9 (dy,dx) taps of an M tile [p0, p0+M) are
// the contiguous slab [p0 + dz*D^2, p0 + dz*D^2 + M + 2D + 2).  The producer
// copies that slab once per (dz, K group) with 1-D bulk copies into shared
// memory as [chunk][row][16 B]; in that arrangement an operand shifted by s
// rows is the same memory with the start address moved by 16*s bytes, which
// is exactly what the no-swizzle K-major tcgen05 descriptor expresses
// (LBO = slab rows * 16 between K core matrices, SBO = 128 between 8-row
// groups).  So each slab feeds 9 taps without re-staging.
//
// Roles (192 threads, one persistent CTA per SM walking the tiles):
//   warp 0 lane 0: producer (cp.async.bulk + mbarrier expect_tx), continuous
//                  across tile boundaries
//   warp 1 lane 0: MMA issuer (tcgen05.mma into one of two TMEM accumulator
//                  buffers), TMEM owner
//   warps 2-5    : epilogue (tcgen05.ld, bias, ReLU, convert, store) of the
//                  other buffer while the next tile accumulates
// Every wait is bounded; a wait that runs out raises the device error word and
// the CTA drains its in-flight copies, frees TMEM and exits.
#include <cuda.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace tdm {
namespace {

constexpr int NSA = 2;      // A slab stages (convolutions)
constexpr int MAX_NSA = 6;  // A stages of a plain GEMM (conv8, feat, MNN distances): 16 KB each
constexpr int MAX_NSB = 12;  // B (weight) stages, sized from the shared-memory budget
constexpr int kThreads = 192;  // warp 0 producer, warp 1 MMA + TMEM owner, warps 2-5 epilogue
constexpr size_t kSmemLimit = 227 * 1024;
constexpr size_t kSmemReserve = 512;  // barriers + TMEM address
constexpr uint64_t kWaitBudgetNs = 500ull * 1000ull * 1000ull;

struct KParams {
  const uint8_t* act;
  int64_t act_cs;
  int64_t rows;
  const uint8_t* wpk;
  const float* bias;
  const float* wscale;
  float in_scale;
  float out_qinv;
  uint8_t* out;
  int64_t out_cs;
  uint8_t* out2;  // CTA-pair conv2 with the y-pair max: the pooled rows (out's chunk stride)
  int D, Do, nz, nyx, kgroups, cpg, cout, out_mode, relu, R, nsa, nsb, ntiles;
  int ksplit;   // K splits of a GEMM (tiles ordered m, n, split); > 1: raw FP32 partials to part
  float* part;  // [ksplit][rows][cout] when ksplit > 1
  int64_t total_tiles;
  int* err;
};

__host__ __device__ constexpr uint32_t tmem_cols_for(int c) {
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

__device__ __forceinline__ bool aborted(const int* err) { return *reinterpret_cast<const volatile int*>(err) != 0; }

// wait_or_flag for barriers the other CTA of a pair arrives on (acquire at
// cluster scope).
__device__ __forceinline__ bool wait_or_flag_cluster(uint32_t bar, uint32_t parity, int* err, int code) {
  if (ptx::mbar_try_wait_cluster(bar, parity)) return true;
  uint64_t t0 = ptx::globaltimer_ns();
  uint32_t spins = 0;
  while (true) {
    if (ptx::mbar_try_wait_cluster(bar, parity)) return true;
    if ((++spins & 255u) == 0) {
      if (aborted(err)) return false;
      if (ptx::globaltimer_ns() - t0 > kWaitBudgetNs) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}

// Waits for phase `parity` of `bar`.  Gives up (false) when another role of
// the kernel has raised the error word, or after budget_ns of wall time, when
// it raises the word with `code` itself.
__device__ __forceinline__ bool wait_or_flag(uint32_t bar, uint32_t parity, int* err, int code,
                                             uint64_t budget_ns = kWaitBudgetNs) {
  if (ptx::mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = ptx::globaltimer_ns();
  uint32_t spins = 0;
  while (true) {
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if ((++spins & 255u) == 0) {
      if (aborted(err)) return false;
      if (ptx::globaltimer_ns() - t0 > budget_ns) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}

#ifdef TDM_WAIT_STATS
// Diagnostic build only: cycles spent in each kind of wait, summed over CTAs.
// slots: 0 MMA<-accEmpty, 1 MMA<-fullA, 2 MMA<-fullB, 3 producer<-emptyA,
//        4 producer<-emptyB, 5 epilogue<-accFull, 6 MMA loop total, 7 producer loop total
//        (grid and dx-fused kernels); 8..15 the same for the gathered-row kernel,
//        with 11 = gather warps <- emptyA and 15 = gather loop total
__device__ unsigned long long g_wait_stats[16];
#define TDM_TIMED_WAIT(slot, expr)                                           \
  ([&]() {                                                                   \
    long long _c0 = clock64();                                               \
    bool _r = (expr);                                                        \
    atomicAdd(&g_wait_stats[slot], (unsigned long long)(clock64() - _c0));   \
    return _r;                                                               \
  }())
#else
#define TDM_TIMED_WAIT(slot, expr) (expr)
#endif

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// An M tile has no valid output row when it lies past the last input row or
// entirely in the z >= Do tail of one patch (those tiles are skipped by every
// role alike).
__device__ __forceinline__ bool tile_has_work(const KParams& p, int64_t m0, int mcta) {
  if (m0 >= p.rows) return false;
  if (p.nyx == 1) return true;
  const int64_t D2 = (int64_t)p.D * p.D, D3 = D2 * p.D;
  // 32-bit remainder when the row index fits (every tile loop calls this)
  const int64_t r0 = p.rows <= INT32_MAX ? (int64_t)((uint32_t)m0 % (uint32_t)D3) : m0 % D3;
  return !(r0 >= (int64_t)p.Do * D2 && r0 + mcta <= D3);
}

// a / d for row indices: 32-bit unsigned division when the layer's rows fit
__device__ __forceinline__ int64_t row_div(int64_t a, int d, bool rows32) {
  return rows32 ? (int64_t)((uint32_t)a / (uint32_t)d) : a / d;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 t = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&t);
}

__device__ __forceinline__ uint32_t pack_e4m3x4(float a, float b, float c, float d) {
  uint32_t lo;
  asm("{\n\t.reg .b16 l, h;\n\t"
      "cvt.rn.satfinite.e4m3x2.f32 l, %2, %1;\n\t"
      "cvt.rn.satfinite.e4m3x2.f32 h, %4, %3;\n\t"
      "mov.b32 %0, {l, h};\n\t}"
      : "=r"(lo)
      : "f"(a), "f"(b), "f"(c), "f"(d));
  return lo;
}

// 16 consecutive floats (16-byte aligned) as four vector loads.
__device__ __forceinline__ void load16(const float* p, float (&v)[16]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 c = __ldg(reinterpret_cast<const float4*>(p) + k);
    v[4 * k] = c.x;
    v[4 * k + 1] = c.y;
    v[4 * k + 2] = c.z;
    v[4 * k + 3] = c.w;
  }
}

// Persistent, warp-specialised implicit-GEMM convolution.  Each CTA walks the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...; the load pipeline runs across
// tile boundaries and the TMEM accumulator is double-buffered, so the epilogue
// of one tile overlaps the MMAs of the next.
template <int NT, int MSUB, bool FP8_IN, bool FP8_OUT>
__global__ void __launch_bounds__(kThreads, 1) tc_conv_kernel(const KParams p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int MCTA = MSUB * 128;
  constexpr uint32_t ACC_COLS = MSUB * NT;  // one accumulator buffer
  constexpr uint32_t TMEM_COLS = tmem_cols_for(2 * ACC_COLS);
  static_assert(2 * ACC_COLS <= 512, "two accumulator buffers must fit in TMEM");
  const int R = p.R, nsb = p.nsb;
  const uint32_t a_stage = 16u * (uint32_t)p.cpg * (uint32_t)R;
  constexpr uint32_t b_stage = NT * 128u;
  uint8_t* sA = smem;
  const int nsa = p.nsa;  // A stages (more for plain GEMMs, whose stages are small)
  uint8_t* sB = smem + nsa * a_stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + (size_t)nsb * b_stage);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * MAX_NSA + 2 * MAX_NSB + 5);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!__syncthreads_and(aborted(p.err) ? 0 : 1)) return;  // another CTA already failed

  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * MAX_NSA;
  const uint32_t fullB = emptyA + 8 * MAX_NSA, emptyB = fullB + 8 * MAX_NSB;
  const uint32_t accFull = emptyB + 8 * MAX_NSB, accEmpty = accFull + 16, done = accEmpty + 16;
  if (threadIdx.x == 0) {
    for (int i = 0; i < nsa; ++i) { ptx::mbar_init(fullA + 8 * i, 1); ptx::mbar_init(emptyA + 8 * i, 1); }
    for (int i = 0; i < nsb; ++i) { ptx::mbar_init(fullB + 8 * i, 1); ptx::mbar_init(emptyB + 8 * i, 1); }
    for (int i = 0; i < 2; ++i) { ptx::mbar_init(accFull + 8 * i, 1); ptx::mbar_init(accEmpty + 8 * i, 4); }
    ptx::mbar_init(done, 1);
    ptx::fence_barrier_init();
    ptx::fence_proxy_async_smem();
  }
  if (warp == 1) {
    ptx::tmem_alloc(ptx::smem_u32(tmem_holder), TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t sA_u = ptx::smem_u32(sA), sB_u = ptx::smem_u32(sB);
  const int64_t plane = (int64_t)p.D * p.D;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- producer ----------------
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      int sa = 0, sb = 0;
      uint32_t pha = 0, phb = 0;
      int armedA[MAX_NSA], armedB[MAX_NSB];  // parity of each stage's last arming, -1 = never
      for (int i = 0; i < MAX_NSA; ++i) armedA[i] = -1;
      for (int i = 0; i < MAX_NSB; ++i) armedB[i] = -1;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t / ((int64_t)p.ntiles * p.ksplit)) * MCTA;
        const int nt = (int)((t / p.ksplit) % p.ntiles);
        const int kg = p.kgroups / p.ksplit, cg0 = (int)(t % p.ksplit) * kg;
        if (!tile_has_work(p, m0, MCTA)) continue;
        for (int zt = 0; zt < p.nz && ok; ++zt) {
          for (int cg = cg0; cg < cg0 + kg && ok; ++cg) {
            if (!TDM_TIMED_WAIT(3, wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
            ptx::mbar_arrive_expect_tx(fullA + 8 * sa, a_stage);
            armedA[sa] = (int)pha;
            const uint8_t* src = p.act + (int64_t)cg * p.cpg * p.act_cs + (m0 + zt * plane) * 16;
            for (int j = 0; j < p.cpg; ++j)
              ptx::bulk_g2s(sA_u + sa * a_stage + j * R * 16, src + j * p.act_cs, R * 16, fullA + 8 * sa);
            if (++sa == nsa) { sa = 0; pha ^= 1; }
            for (int yx = 0; yx < p.nyx; ++yx) {
              if (!TDM_TIMED_WAIT(4, wait_or_flag(emptyB + 8 * sb, phb ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
              ptx::mbar_arrive_expect_tx(fullB + 8 * sb, b_stage);
              armedB[sb] = (int)phb;
              const int64_t blk = (((int64_t)nt * p.nz + zt) * p.kgroups + cg) * p.nyx + yx;
              ptx::bulk_g2s(sB_u + sb * b_stage, p.wpk + blk * b_stage, b_stage, fullB + 8 * sb);
              if (++sb == nsb) { sb = 0; phb ^= 1; }
            }
          }
        }
      }
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[7], (unsigned long long)(clock64() - t_loop0));
#endif
      // Drain: every armed stage must have landed before the CTA can exit.
      for (int i = 0; i < nsa; ++i)
        if (armedA[i] >= 0) wait_or_flag(fullA + 8 * i, (uint32_t)armedA[i], p.err, DEV_TIMEOUT_PRODUCER);
      for (int i = 0; i < nsb; ++i)
        if (armedB[i] >= 0) wait_or_flag(fullB + 8 * i, (uint32_t)armedB[i], p.err, DEV_TIMEOUT_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      constexpr uint32_t idesc = FP8_IN ? ptx::make_idesc(NT, 128, 0, 0) : ptx::make_idesc(NT, 128, 1, 1);
      int sa = 0, sb = 0;
      uint32_t pha = 0, phb = 0;
      bool ok = true;
      const uint32_t lboA = (uint32_t)R * 16u;
      const uint64_t aDesc0 = ptx::smem_desc(sA_u, lboA, 128), bDesc0 = ptx::smem_desc(sB_u, NT * 16, 128);
      uint32_t j = 0;  // tiles done by this CTA
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t / ((int64_t)p.ntiles * p.ksplit)) * MCTA;
        const int kg = p.kgroups / p.ksplit;
        if (!tile_has_work(p, m0, MCTA)) continue;
        const uint32_t buf = j & 1u, use = j >> 1;
        if (!TDM_TIMED_WAIT(0, wait_or_flag(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * ACC_COLS;
        uint32_t accumulate = 0;
        for (int zt = 0; zt < p.nz && ok; ++zt) {
          for (int cg = 0; cg < kg && ok; ++cg) {
            if (!TDM_TIMED_WAIT(1, wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
            ptx::tc_fence_after();
            const uint64_t aStage = ptx::desc_advance(aDesc0, sa * a_stage);
            for (int yx = 0; yx < p.nyx; ++yx) {
              if (!TDM_TIMED_WAIT(2, wait_or_flag(fullB + 8 * sb, phb, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
              ptx::tc_fence_after();
              const uint64_t bStage = ptx::desc_advance(bDesc0, sb * b_stage);
              const int off = (p.nyx > 1) ? (yx / 3) * p.D + (yx % 3) : 0;
              const uint64_t aTap = ptx::desc_advance(aStage, (uint32_t)off * 16u);
#pragma unroll 4
              for (int kk = 0; kk < p.cpg / 2; ++kk) {
                const uint64_t bdesc = ptx::desc_advance(bStage, (2 * kk) * NT * 16);
#pragma unroll
                for (int i = 0; i < MSUB; ++i) {
                  const uint64_t adesc = ptx::desc_advance(aTap, (2 * kk) * lboA + (uint32_t)(i * 128) * 16u);
                  if (FP8_IN) ptx::mma_f8(dbase + i * NT, adesc, bdesc, idesc, accumulate);
                  else ptx::mma_f16(dbase + i * NT, adesc, bdesc, idesc, accumulate);
                }
                accumulate = 1;
              }
              ptx::mma_commit(emptyB + 8 * sb);
              if (++sb == nsb) { sb = 0; phb ^= 1; }
            }
            ptx::mma_commit(emptyA + 8 * sa);
            if (++sa == nsa) { sa = 0; pha ^= 1; }
          }
        }
        ptx::mma_commit(accFull + 8 * buf);  // fires when this tile's MMAs are complete
        ++j;
      }
      ptx::mma_commit(done);
      wait_or_flag(done, 0, p.err, DEV_TIMEOUT_MMA);
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[6], (unsigned long long)(clock64() - t_loop0));
#endif
    }
  } else {
    // ---------------- epilogue (warps 2-5: TMEM lane quarter warp % 4) ----------------
    const int q = warp & 3;
    const int64_t D3 = (int64_t)p.D * p.D * p.D;
    uint32_t j = 0;
    for (int64_t t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
      const int64_t m0 = (t / ((int64_t)p.ntiles * p.ksplit)) * MCTA;
      const int n0 = (int)((t / p.ksplit) % p.ntiles) * NT;
      const int ks = (int)(t % p.ksplit);
      if (!tile_has_work(p, m0, MCTA)) continue;
      const uint32_t buf = j & 1u, use = j >> 1;
      const bool have =
          __all_sync(0xffffffffu,
                     TDM_TIMED_WAIT(5, wait_or_flag(accFull + 8 * buf, use & 1u, p.err, DEV_TIMEOUT_EPILOGUE)) ? 1 : 0) != 0;
      if (!have) break;
      ptx::tc_fence_after();
#pragma unroll 1
      for (int i = 0; i < MSUB; ++i) {
        const int64_t row = m0 + i * 128 + q * 32 + lane;
        bool valid = row < p.rows;
        int64_t b = 0, pout = row;
        int x = 0, y = 0, z = 0;
        if (p.nyx > 1 && valid) {
          b = row / D3;
          int r = (int)(row - b * D3);
          z = r / (p.D * p.D);
          y = (r / p.D) % p.D;
          x = r % p.D;
          valid = x < p.Do && y < p.Do && z < p.Do;
          pout = ((b * p.Do + z) * p.Do + y) * p.Do + x;
        }
#pragma unroll 1
        for (int c0 = 0; c0 < NT; c0 += 16) {
          float v[16];
          ptx::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_COLS + (uint32_t)(i * NT + c0), v);
          if (!valid) continue;
          const int n = n0 + c0;
          if (p.ksplit > 1) {  // raw partial sums; splitk_reduce_kernel finishes the layer
            float4* dst = reinterpret_cast<float4*>(p.part + ((int64_t)ks * p.rows + row) * p.cout + n);
#pragma unroll
            for (int h = 0; h < 4; ++h) dst[h] = make_float4(v[4 * h], v[4 * h + 1], v[4 * h + 2], v[4 * h + 3]);
            continue;
          }
          float bs[16], sc[16];
          load16(p.bias + n, bs);
          if (FP8_IN) load16(p.wscale + n, sc);
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            float a = v[e];
            if (FP8_IN) a = a * (p.in_scale * sc[e]);
            a += bs[e];
            if (p.relu) a = fmaxf(a, 0.0f);
            v[e] = a;
          }
          if (p.out_mode == TC_OUT_F32_ROWS) {
            float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(p.out) + row * p.cout + n);
#pragma unroll
            for (int h = 0; h < 4; ++h) dst[h] = make_float4(v[4 * h], v[4 * h + 1], v[4 * h + 2], v[4 * h + 3]);
            continue;
          }
          if (FP8_OUT) {
            uint4 o;
            o.x = pack_e4m3x4(v[0] * p.out_qinv, v[1] * p.out_qinv, v[2] * p.out_qinv, v[3] * p.out_qinv);
            o.y = pack_e4m3x4(v[4] * p.out_qinv, v[5] * p.out_qinv, v[6] * p.out_qinv, v[7] * p.out_qinv);
            o.z = pack_e4m3x4(v[8] * p.out_qinv, v[9] * p.out_qinv, v[10] * p.out_qinv, v[11] * p.out_qinv);
            o.w = pack_e4m3x4(v[12] * p.out_qinv, v[13] * p.out_qinv, v[14] * p.out_qinv, v[15] * p.out_qinv);
            int64_t chunk, prow;
            if (p.out_mode == TC_OUT_C8_TAPS) {
              chunk = (int64_t)((z * p.Do + y) * p.Do + x) * (p.cout / 16) + n / 16;
              prow = b;
            } else {
              chunk = n / 16;
              prow = pout;
            }
            *reinterpret_cast<uint4*>(p.out + chunk * p.out_cs + prow * 16) = o;
          } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              uint4 o;
              o.x = pack_bf16x2(v[8 * h + 0], v[8 * h + 1]);
              o.y = pack_bf16x2(v[8 * h + 2], v[8 * h + 3]);
              o.z = pack_bf16x2(v[8 * h + 4], v[8 * h + 5]);
              o.w = pack_bf16x2(v[8 * h + 6], v[8 * h + 7]);
              int64_t chunk, prow;
              if (p.out_mode == TC_OUT_C8_TAPS) {
                chunk = (int64_t)((z * p.Do + y) * p.Do + x) * (p.cout / 8) + n / 8 + h;
                prow = b;
              } else {
                chunk = n / 8 + h;
                prow = pout;
              }
              *reinterpret_cast<uint4*>(p.out + chunk * p.out_cs + prow * 16) = o;
            }
          }
        }
      }
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(accEmpty + 8 * buf);
      ++j;
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Split-K GEMM finish: out = act(sum_s part[s] (s in order) * scale + bias) for
// 8 channels of one row per thread, in the layer's output format.
template <bool FP8_IN>
__global__ __launch_bounds__(256) void splitk_reduce_kernel(const float* __restrict__ part, int ksplit, int64_t rows,
                                                            int cout, const float* __restrict__ bias,
                                                            const float* __restrict__ wscale, float in_scale, int relu,
                                                            int out_mode, uint8_t* __restrict__ out, int64_t out_cs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int groups = cout / 8;
  if (i >= rows * groups) return;
  const int64_t row = i / groups;
  const int n = (int)(i - row * groups) * 8;
  float v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = 0.0f;
  for (int k = 0; k < ksplit; ++k) {
    const float4* src = reinterpret_cast<const float4*>(part + ((int64_t)k * rows + row) * cout + n);
    const float4 a = __ldg(src), b = __ldg(src + 1);
    v[0] += a.x; v[1] += a.y; v[2] += a.z; v[3] += a.w;
    v[4] += b.x; v[5] += b.y; v[6] += b.z; v[7] += b.w;
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    float a = v[e];
    if (FP8_IN) a = a * (in_scale * __ldg(wscale + n + e));
    a += __ldg(bias + n + e);
    if (relu) a = fmaxf(a, 0.0f);
    v[e] = a;
  }
  if (out_mode == TC_OUT_F32_ROWS) {
    float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(out) + row * cout + n);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  } else {  // TC_OUT_C8_ROWS: BF16 chunk n / 8, row = input row
    uint4 o;
    o.x = pack_bf16x2(v[0], v[1]);
    o.y = pack_bf16x2(v[2], v[3]);
    o.z = pack_bf16x2(v[4], v[5]);
    o.w = pack_bf16x2(v[6], v[7]);
    *reinterpret_cast<uint4*>(out + (int64_t)(n / 8) * out_cs + row * 16) = o;
  }
}

// ---------------------------------------------------------------------------
// Gathered-row form of a 3x3x3 conv (conv3..conv7).
//
// The grid form above computes a GEMM row for every input position and drops
// the rows with x, y or z >= Do in its epilogue: 1.65x (conv3) to 4.6x (conv7)
// the useful MACs.  Here M runs over the valid output positions only, row
// m = ((b*Do + z)*Do + y)*Do + x, and four gather warps build each tap's A
// operand row by row: the 16-byte chunks of input position
// ((b*D + z+dz)*D + y+dy)*D + x+dx go by cp.async straight into the K-major
// stage layout [chunk][row][16 B].  A stage is one (tap, K group).  The weight
// stages (the grid form's packing), the MMA issue and the TMEM epilogue are the
// grid form's, and taps and K groups run in the same order, so every output is
// the same sum taken in the same order.
// ---------------------------------------------------------------------------
constexpr int kGWarps = 4;                          // gather warps (warps 6..9)
// warps 10..13: a second set of epilogue warps (each lane quarter drains its
// accumulator in two column halves), so a single-buffered tile frees TMEM sooner
constexpr int kGThreads = kThreads + 32 * kGWarps + 128;
constexpr int kGNSA = 4;                            // A stages (gathered rows)
constexpr int kXNSA = 3;                            // A stages (x runs: three B stages per A stage)

// 16-byte global -> shared copy; src_bytes = 0 writes zeros without reading.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int NT, int MSUB, bool FP8, bool XRUN, bool WT>
__global__ void __launch_bounds__(kGThreads, 1) tc_conv_gather_kernel(const KParams p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int MCTA = MSUB * 128;
  // WT (weights as the A operand, 128 output channels): one M = 128 (channels)
  // x N = MCTA (rows) MMA per K step instead of MSUB M = 128 (rows) x N = 128
  // ones -- 12 KB of operands per 524k MACs instead of 16 KB.  The accumulator
  // then holds one channel per TMEM lane and the epilogue transposes through
  // shared memory.
  static_assert(!WT || NT == 128, "weights-as-A form: 128 output channels");
  constexpr uint32_t ACC_COLS = WT ? MCTA : MSUB * NT;
  constexpr int NBUF = 2 * ACC_COLS <= 512 ? 2 : 1;  // accumulator buffers
  constexpr uint32_t TMEM_COLS = tmem_cols_for(NBUF * ACC_COLS);
  static_assert(ACC_COLS <= 512, "the accumulator must fit in TMEM");
  constexpr int E = FP8 ? 16 : 8;  // channels per 16-byte chunk
  constexpr int NSA = XRUN ? kXNSA : kGNSA;  // A stages
  constexpr int DEPTH = NSA - 1;              // stages a gather thread keeps in flight
  constexpr int RS = MCTA + (XRUN ? 8 : 0);   // rows per A stage (x-run form: +2 for the dx shifts, padded)
  const int nsb = p.nsb, cpg = p.cpg;
  const uint32_t a_stage = 16u * (uint32_t)cpg * RS;
  constexpr uint32_t b_stage = NT * 128u;
  uint8_t* sB = smem + NSA * a_stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + (size_t)nsb * b_stage);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * NSA + 2 * MAX_NSB + 5);
  // WT epilogue transposition tiles: per epilogue warp (8) 16 rows x 32 channels of BF16
  uint16_t* sT = reinterpret_cast<uint16_t*>(
      (reinterpret_cast<uintptr_t>(tmem_holder + 4) + 15) & ~static_cast<uintptr_t>(15));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!__syncthreads_and(aborted(p.err) ? 0 : 1)) return;  // another CTA already failed

  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * NSA;
  const uint32_t fullB = emptyA + 8 * NSA, emptyB = fullB + 8 * MAX_NSB;
  const uint32_t accFull = emptyB + 8 * MAX_NSB, accEmpty = accFull + 16, done = accEmpty + 16;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NSA; ++i) {
      ptx::mbar_init(fullA + 8 * i, 32 * kGWarps);  // every gather thread arrives
      ptx::mbar_init(emptyA + 8 * i, 1);
    }
    for (int i = 0; i < nsb; ++i) { ptx::mbar_init(fullB + 8 * i, 1); ptx::mbar_init(emptyB + 8 * i, 1); }
    for (int i = 0; i < 2; ++i) { ptx::mbar_init(accFull + 8 * i, 1); ptx::mbar_init(accEmpty + 8 * i, 8); }
    ptx::mbar_init(done, 1);
    ptx::fence_barrier_init();
    ptx::fence_proxy_async_smem();
  }
  if (warp == 1) {
    ptx::tmem_alloc(ptx::smem_u32(tmem_holder), TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t sA_u = ptx::smem_u32(smem), sB_u = ptx::smem_u32(sB);
  const int Do2 = p.Do * p.Do, Do3 = Do2 * p.Do;
  const int Dx = XRUN ? p.D : p.Do;  // x extent of the M rows

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- weight producer ----------------
      int sb = 0;
      uint32_t phb = 0;
      int armedB[MAX_NSB];
      for (int i = 0; i < MAX_NSB; ++i) armedB[i] = -1;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int nt = (int)(t % p.ntiles);
        for (int zt = 0; zt < p.nz && ok; ++zt)
          for (int cg = 0; cg < p.kgroups && ok; ++cg)
            for (int yx = 0; yx < p.nyx; ++yx) {
              if (!TDM_TIMED_WAIT(12, wait_or_flag(emptyB + 8 * sb, phb ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
              ptx::mbar_arrive_expect_tx(fullB + 8 * sb, b_stage);
              armedB[sb] = (int)phb;
              const int64_t blk = (((int64_t)nt * p.nz + zt) * p.kgroups + cg) * p.nyx + yx;
              ptx::bulk_g2s(sB_u + sb * b_stage, p.wpk + blk * b_stage, b_stage, fullB + 8 * sb);
              if (++sb == nsb) { sb = 0; phb ^= 1; }
            }
      }
      for (int i = 0; i < nsb; ++i)
        if (armedB[i] >= 0) wait_or_flag(fullB + 8 * i, (uint32_t)armedB[i], p.err, DEV_TIMEOUT_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      constexpr uint32_t idesc = WT ? (FP8 ? ptx::make_idesc(MCTA, 128, 0, 0) : ptx::make_idesc(MCTA, 128, 1, 1))
                                    : (FP8 ? ptx::make_idesc(NT, 128, 0, 0) : ptx::make_idesc(NT, 128, 1, 1));
      constexpr uint32_t lboA = RS * 16u;
      const uint64_t aDesc0 = ptx::smem_desc(sA_u, lboA, 128), bDesc0 = ptx::smem_desc(sB_u, NT * 16, 128);
      int sa = 0, sb = 0;
      uint32_t pha = 0, phb = 0;
      bool ok = true;
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      uint32_t j = 0;  // tiles done by this CTA
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const uint32_t buf = j % NBUF, use = j / NBUF;
        if (!TDM_TIMED_WAIT(8, wait_or_flag(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA))) break;
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * ACC_COLS;
        uint32_t accumulate = 0;
        // A stage per (dz, K group, tap) -- or per (dz, K group, dy) in the
        // x-run form, where the three dx taps read it shifted by dx rows
        constexpr int TAPS_PER_A = XRUN ? 3 : 1;
        for (int zt = 0; zt < p.nz && ok; ++zt)
          for (int cg = 0; cg < p.kgroups && ok; ++cg)
            for (int ya = 0; ya < p.nyx / TAPS_PER_A && ok; ++ya) {
              if (!TDM_TIMED_WAIT(9, wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
              const uint64_t aStage = ptx::desc_advance(aDesc0, sa * a_stage);
              for (int dx = 0; dx < TAPS_PER_A; ++dx) {
                if (!TDM_TIMED_WAIT(10, wait_or_flag(fullB + 8 * sb, phb, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
                ptx::tc_fence_after();
                const uint64_t bStage = ptx::desc_advance(bDesc0, sb * b_stage);
                const uint64_t aTap = ptx::desc_advance(aStage, (uint32_t)dx * 16u);
#pragma unroll 4
                for (int kk = 0; kk < cpg / 2; ++kk) {
                  const uint64_t wdesc = ptx::desc_advance(bStage, (2 * kk) * NT * 16);
                  if (WT) {  // D[channel][row] += W[channel][k] . X[row][k]
                    const uint64_t xdesc = ptx::desc_advance(aTap, (2 * kk) * lboA);
                    if (FP8) ptx::mma_f8(dbase, wdesc, xdesc, idesc, accumulate);
                    else ptx::mma_f16(dbase, wdesc, xdesc, idesc, accumulate);
                  } else {
#pragma unroll
                    for (int i = 0; i < MSUB; ++i) {
                      const uint64_t adesc = ptx::desc_advance(aTap, (2 * kk) * lboA + (uint32_t)(i * 128) * 16u);
                      if (FP8) ptx::mma_f8(dbase + i * NT, adesc, wdesc, idesc, accumulate);
                      else ptx::mma_f16(dbase + i * NT, adesc, wdesc, idesc, accumulate);
                    }
                  }
                  accumulate = 1;
                }
                ptx::mma_commit(emptyB + 8 * sb);
                if (++sb == nsb) { sb = 0; phb ^= 1; }
              }
              ptx::mma_commit(emptyA + 8 * sa);
              if (++sa == NSA) { sa = 0; pha ^= 1; }
            }
        ptx::mma_commit(accFull + 8 * buf);  // fires when this tile's MMAs are complete
        ++j;
      }
      ptx::mma_commit(done);
      wait_or_flag(done, 0, p.err, DEV_TIMEOUT_MMA);
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[14], (unsigned long long)(clock64() - t_loop0));
#endif
    }
  } else if (warp < 6 || warp >= 10) {
    // ---------------- epilogue (warps 2-5 and 10-13: TMEM lane quarter warp % 4,
    // column half eh) ----------------
    const int q = warp & 3, eh = warp >= 10 ? 1 : 0;
    const bool rows32 = p.rows <= INT32_MAX;
    uint32_t j = 0;
    for (int64_t t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
      const int64_t m0 = (t / p.ntiles) * MCTA;
      const int n0 = (int)(t % p.ntiles) * NT;
      const uint32_t buf = j % NBUF, use = j / NBUF;
      const bool have =
          __all_sync(0xffffffffu, TDM_TIMED_WAIT(13, wait_or_flag(accFull + 8 * buf, use & 1u, p.err, DEV_TIMEOUT_EPILOGUE)) ? 1 : 0) != 0;
      if (!have) break;
      ptx::tc_fence_after();
      if constexpr (WT) {
        // lane = output channel n0 + 32 q + lane; columns = the tile's rows
        const int c = n0 + q * 32 + lane;
        const float bias_c = __ldg(p.bias + c);
        const float scale_c = FP8 ? p.in_scale * __ldg(p.wscale + c) : 1.0f;
        uint16_t* tw = sT + (eh * 4 + q) * (16 * 32);      // BF16: [row][channel] halves
        uint8_t* tb = reinterpret_cast<uint8_t*>(tw);      // E4M3: [row][channel] bytes
#pragma unroll 1
        for (int c1 = eh * (MCTA / 2); c1 < (eh + 1) * (MCTA / 2); c1 += 16) {
          float v[16];
          ptx::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_COLS + (uint32_t)c1, v);
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            float a = v[e];
            if (FP8) a = a * scale_c;
            a += bias_c;
            if (p.relu) a = fmaxf(a, 0.0f);
            v[e] = a;
          }
          if (FP8) {
#pragma unroll
            for (int e = 0; e < 16; e += 2) {
              uint16_t pr;
              asm("cvt.rn.satfinite.e4m3x2.f32 %0, %2, %1;" : "=h"(pr) : "f"(v[e] * p.out_qinv), "f"(v[e + 1] * p.out_qinv));
              tb[e * 32 + lane] = (uint8_t)(pr & 0xFFu);
              tb[(e + 1) * 32 + lane] = (uint8_t)(pr >> 8);
            }
          } else {
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const __nv_bfloat16 h = __float2bfloat16_rn(v[e]);
              tw[e * 32 + lane] = *reinterpret_cast<const uint16_t*>(&h);
            }
          }
          __syncwarp();
          // 16 rows x (BF16: 4 chunks of 8 channels, two per lane; E4M3: 2 chunks of 16, one per lane)
          constexpr int PER_LANE = FP8 ? 1 : 2;
#pragma unroll
          for (int k2 = 0; k2 < PER_LANE; ++k2) {
            const int id = lane + 32 * k2;
            const int rr = FP8 ? (id >> 1) : (id >> 2), ch = FP8 ? (id & 1) : (id & 3);
            const int64_t row = m0 + c1 + rr;
            bool valid = row < p.rows;
            int64_t pos;
            if (XRUN) {
              const int64_t yz = row_div(row, Dx, rows32);
              const int x = (int)(row - yz * Dx);
              valid = valid && x < p.Do;
              pos = yz * p.Do + x;  // ((b*Do + z)*Do + y)*Do + x
            } else {
              pos = row;
            }
            const uint4 val = FP8 ? *reinterpret_cast<const uint4*>(tb + rr * 32 + ch * 16)
                                  : *reinterpret_cast<const uint4*>(tw + rr * 32 + ch * 8);
            const int64_t chunk = FP8 ? (n0 / 16 + q * 2 + ch) : (n0 / 8 + q * 4 + ch);
            if (valid) *reinterpret_cast<uint4*>(p.out + chunk * p.out_cs + pos * 16) = val;
          }
          __syncwarp();
        }
      } else {
#pragma unroll 1
      for (int i = 0; i < MSUB; ++i) {
        const int64_t row = m0 + i * 128 + q * 32 + lane;
        bool valid = row < p.rows;
        int64_t b, pos;  // patch, output position (row of the next layer's grid)
        int tap;         // output position within the patch
        if (XRUN) {      // rows (b, z, y, x < D): outputs where x < Do
          const int64_t yz = row_div(row, Dx, rows32);
          const int x = (int)(row - yz * Dx);
          valid = valid && x < p.Do;
          b = row_div(yz, Do2, rows32);
          tap = (int)(yz - b * Do2) * p.Do + x;
        } else {
          b = row_div(row, Do3, rows32);
          tap = (int)(row - b * Do3);
        }
        pos = b * Do3 + tap;
#pragma unroll 1
        for (int c1 = eh * (NT / 2); c1 < (eh + 1) * (NT / 2); c1 += 32) {
          uint32_t r2[2][16];  // 32 accumulator columns: two loads, one wait
          const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_COLS + (uint32_t)(i * NT + c1);
          ptx::tmem_ld16_nowait(ta, r2[0]);
          ptx::tmem_ld16_nowait(ta + 16, r2[1]);
          ptx::tmem_wait_ld();
          if (!valid) continue;
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
          float v[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(r2[hh][e]);
          const int n = n0 + c1 + 16 * hh;
          float bs[16], sc[16];
          load16(p.bias + n, bs);
          if (FP8) load16(p.wscale + n, sc);
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            float a = v[e];
            if (FP8) a = a * (p.in_scale * sc[e]);
            a += bs[e];
            if (p.relu) a = fmaxf(a, 0.0f);
            v[e] = a;
          }
          // chunk-planar output: next layer's input grid (row = position) or
          // conv8's operand (chunk = tap * Cout/E + channel chunk, row = patch)
          const bool taps = p.out_mode == TC_OUT_C8_TAPS;
          const int64_t chunk0 = (taps ? (int64_t)tap * (p.cout / E) : 0) + n / E;
          const int64_t prow = taps ? b : pos;
          if (FP8) {
            uint4 o;
            o.x = pack_e4m3x4(v[0] * p.out_qinv, v[1] * p.out_qinv, v[2] * p.out_qinv, v[3] * p.out_qinv);
            o.y = pack_e4m3x4(v[4] * p.out_qinv, v[5] * p.out_qinv, v[6] * p.out_qinv, v[7] * p.out_qinv);
            o.z = pack_e4m3x4(v[8] * p.out_qinv, v[9] * p.out_qinv, v[10] * p.out_qinv, v[11] * p.out_qinv);
            o.w = pack_e4m3x4(v[12] * p.out_qinv, v[13] * p.out_qinv, v[14] * p.out_qinv, v[15] * p.out_qinv);
            *reinterpret_cast<uint4*>(p.out + chunk0 * p.out_cs + prow * 16) = o;
          } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              uint4 o;
              o.x = pack_bf16x2(v[8 * h + 0], v[8 * h + 1]);
              o.y = pack_bf16x2(v[8 * h + 2], v[8 * h + 3]);
              o.z = pack_bf16x2(v[8 * h + 4], v[8 * h + 5]);
              o.w = pack_bf16x2(v[8 * h + 6], v[8 * h + 7]);
              *reinterpret_cast<uint4*>(p.out + (chunk0 + h) * p.out_cs + prow * 16) = o;
            }
          }
          }
        }
      }
      }  // WT / row-major accumulator
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(accEmpty + 8 * buf);
      ++j;
    }
  } else {
    // ---------------- gather warps: each tap's A rows into the stages ----------------
    const int gt = threadIdx.x - kThreads;  // 0 .. 127: row gt of every 128-row sub-tile
    int sa = 0;
    uint32_t pha = 0;
    int pend[DEPTH];  // stages copied but not yet published, oldest first from q0
    int q0 = 0, np = 0;
    bool ok = true;
    const int64_t plane = (int64_t)p.D * p.D;
    const bool rows32 = p.rows <= INT32_MAX;
#ifdef TDM_WAIT_STATS
    const long long t_loop0 = clock64();
#endif
    for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
      const int64_t m0 = (t / p.ntiles) * MCTA;
      // this thread's stage rows: gt + 128 i, and in the x-run form also the
      // padding row MCTA + gt (gt < 8; the first rows of the next tile)
      constexpr int NR = MSUB + (XRUN ? 1 : 0);
      int64_t base[NR];
      uint32_t bytes[NR];
      int slot[NR];
#pragma unroll
      for (int i = 0; i < NR; ++i) {
        slot[i] = i < MSUB ? i * 128 + gt : MCTA + gt;
        const int64_t row = m0 + slot[i];
        base[i] = 0;
        bytes[i] = 0;  // rows past the end are zero-filled
        if (row < p.rows && (i < MSUB || gt < 8)) {
          const int64_t yz = row_div(row, Dx, rows32);  // (b, z, y)
          const int x = (int)(row - yz * Dx);
          const int64_t b = row_div(yz, Do2, rows32);
          const int r = (int)(yz - b * Do2);
          base[i] = ((b * p.D + r / p.Do) * p.D + r % p.Do) * p.D + x;
          bytes[i] = 16;
        }
      }
      constexpr int TAPS_PER_A = XRUN ? 3 : 1;
      for (int zt = 0; zt < p.nz && ok; ++zt)
        for (int cg = 0; cg < p.kgroups && ok; ++cg)
          for (int ya = 0; ya < p.nyx / TAPS_PER_A; ++ya) {
            if (!TDM_TIMED_WAIT(11, wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
            // tap offset in the input grid (the x-run form stages dx = 0; dx
            // comes from the MMA's row shift)
            const int64_t off = XRUN ? zt * plane + ya * p.D : zt * plane + (ya / 3) * p.D + (ya % 3);
            const uint32_t dst = sA_u + sa * a_stage;
            const uint8_t* cbase = p.act + (int64_t)cg * cpg * p.act_cs;
#pragma unroll
            for (int i = 0; i < NR; ++i) {
              if (i == MSUB && gt >= 8) continue;
              const uint8_t* src = cbase + (base[i] + off) * 16;
#pragma unroll 4
              for (int c = 0; c < cpg; ++c)
                cp_async16(dst + (uint32_t)(c * RS + slot[i]) * 16u, src + c * p.act_cs, bytes[i]);
            }
            cp_async_commit();
            pend[(q0 + np) % DEPTH] = sa;
            if (++np == DEPTH) {  // publish the oldest stage once its copies have landed
              cp_async_wait<DEPTH - 1>();
              ptx::fence_proxy_async_smem();  // generic-proxy writes visible to the tensor core
              mbar_arrive(fullA + 8 * pend[q0]);
              q0 = (q0 + 1) % DEPTH;
              --np;
            }
            if (++sa == NSA) { sa = 0; pha ^= 1; }
          }
    }
#ifdef TDM_WAIT_STATS
    if (gt == 0) atomicAdd(&g_wait_stats[15], (unsigned long long)(clock64() - t_loop0));
#endif
    cp_async_wait<0>();  // no copy may still be in flight when the CTA exits
    ptx::fence_proxy_async_smem();
    for (; np > 0; --np) {
      mbar_arrive(fullA + 8 * pend[q0]);
      q0 = (q0 + 1) % DEPTH;
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// dx-fused form of a 3x3x3 conv with 64 BF16 inputs and 64 outputs (conv2).
//
// An N = 64 MMA reads its A rows (4 KB per 128 x 16) and B (2 KB) from
// shared memory for only 128 x 64 x 16 MACs; at the SM's shared-memory rate
// that caps it well below the tensor pipe.  Here the three dx taps of one
// (dz, dy) share the A operand: B = [W(dz,dy,0) | W(dz,dy,1) | W(dz,dy,2)]
// for nt output channels gives N = 3 nt, and accumulator block dx holds
//   P_dx[r] = sum_{dz,dy} A[r + dz D^2 + dy D] . W(dz,dy,dx)
// so output row m = P_0[m] + P_1[m + 1] + P_2[m + 2].  The epilogue takes the
// +1 / +2 rows from the neighbouring TMEM lanes (warp shuffles, and shared
// memory across the 32-lane quarters); a 128-row sub-tile therefore yields
// 126 outputs.  Each CTA owns one half of the output channels (nt = 32,
// N = 96) for all its tiles, so its 110.6 KB of weights are loaded once and
// stay in shared memory; only the A slabs stream.
// ---------------------------------------------------------------------------
constexpr int kDxfNt = 32;
constexpr int kDxfN = 3 * kDxfNt;
constexpr int kDxfSub = 126;
constexpr uint32_t kDxfBlock = 8u * kDxfN * 16u;       // one (dz, dy): 8 K chunks x 96 rows x 16 B
constexpr uint32_t kDxfWBytes = 9u * kDxfBlock;         // one half's weights
// epilogue lane exchange: per tile parity, sub-tile and lane quarter, lane 0's
// P_1 and P_2 and lane 1's P_2 (32 channels each)
constexpr uint32_t kDxfXchg = 2u * 2u * 4u * 96u * 4u;
// output staging for the bulk stores: [sub-tile][chunk][128 rows][16 B]
constexpr uint32_t kDxfStage = 2u * 4u * 128u * 16u;
constexpr int kDxfNSA = 2;  // A slab stages

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// XPOOL: the epilogue also takes the max of each x pair (the first step of
// the 2x2x2 max-pool that follows conv2) and writes x extent Do/2.  Adjacent x
// are adjacent TMEM lanes, every sub-tile starts and ends on an even x (D, Do,
// 126 and the tile starts are even), and max commutes with the monotonic BF16
// and E4M3 rounding, so the pool's result is the same bits.
template <int MSUB, bool FP8_OUT, bool XPOOL>
__global__ void __launch_bounds__(kThreads, 1) tc_conv_dxf_kernel(const KParams p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int MOUT = MSUB * kDxfSub;
  constexpr uint32_t ACC_COLS = MSUB * kDxfN;
  constexpr uint32_t TMEM_COLS = tmem_cols_for(2 * ACC_COLS);
  static_assert(2 * ACC_COLS <= 512, "two accumulator buffers must fit in TMEM");
  const int R = p.R;
  const uint32_t a_stage = 16u * 8u * (uint32_t)R;
  uint8_t* sW = smem;
  uint8_t* sA = smem + kDxfWBytes;
  float* sX = reinterpret_cast<float*>(sA + kDxfNSA * a_stage);
  uint8_t* sO = reinterpret_cast<uint8_t*>(sX) + kDxfXchg;
  int* sVote = reinterpret_cast<int*>(sO + kDxfStage);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sVote + 8);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * kDxfNSA + 6);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!__syncthreads_and(aborted(p.err) ? 0 : 1)) return;

  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * kDxfNSA;
  const uint32_t wfull = emptyA + 8 * kDxfNSA, accFull = wfull + 8, accEmpty = accFull + 16, done = accEmpty + 16;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kDxfNSA; ++i) { ptx::mbar_init(fullA + 8 * i, 1); ptx::mbar_init(emptyA + 8 * i, 1); }
    ptx::mbar_init(wfull, 1);
    for (int i = 0; i < 2; ++i) { ptx::mbar_init(accFull + 8 * i, 1); ptx::mbar_init(accEmpty + 8 * i, 4); }
    ptx::mbar_init(done, 1);
    ptx::fence_barrier_init();
    ptx::fence_proxy_async_smem();
  }
  if (warp == 1) {
    ptx::tmem_alloc(ptx::smem_u32(tmem_holder), TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t sA_u = ptx::smem_u32(sA), sW_u = ptx::smem_u32(sW);
  const int64_t plane = (int64_t)p.D * p.D;
  // the grid is even, so every tile t of this CTA has t % 2 == blockIdx.x % 2
  const int half = blockIdx.x & 1;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- producer: resident weights once, then A slabs ----------------
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      ptx::mbar_arrive_expect_tx(wfull, kDxfWBytes);
      for (int b = 0; b < 9; ++b)
        ptx::bulk_g2s(sW_u + b * kDxfBlock, p.wpk + (size_t)half * kDxfWBytes + (size_t)b * kDxfBlock, kDxfBlock,
                      wfull);
      int sa = 0;
      uint32_t pha = 0;
      int armedA[kDxfNSA];
      for (int i = 0; i < kDxfNSA; ++i) armedA[i] = -1;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t >> 1) * MOUT;
        if (!tile_has_work(p, m0, MOUT)) continue;
        for (int zt = 0; zt < 3; ++zt) {
          if (!TDM_TIMED_WAIT(3, wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
          ptx::mbar_arrive_expect_tx(fullA + 8 * sa, a_stage);
          armedA[sa] = (int)pha;
          const uint8_t* src = p.act + (m0 + zt * plane) * 16;
          for (int j = 0; j < 8; ++j)
            ptx::bulk_g2s(sA_u + sa * a_stage + j * R * 16, src + j * p.act_cs, R * 16, fullA + 8 * sa);
          if (++sa == kDxfNSA) { sa = 0; pha ^= 1; }
        }
        // the next tile's slabs towards L2 while this one is consumed
        const int64_t tn = t + gridDim.x;
        if (ok && tn < p.total_tiles) {
          const int64_t mn = (tn >> 1) * MOUT;
          if (tile_has_work(p, mn, MOUT))
            for (int zt = 0; zt < 3; ++zt)
              for (int j = 0; j < 8; ++j) ptx::bulk_prefetch_l2(p.act + (mn + zt * plane) * 16 + j * p.act_cs, R * 16);
        }
      }
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[7], (unsigned long long)(clock64() - t_loop0));
#endif
      for (int i = 0; i < kDxfNSA; ++i)
        if (armedA[i] >= 0) wait_or_flag(fullA + 8 * i, (uint32_t)armedA[i], p.err, DEV_TIMEOUT_PRODUCER);
      wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      constexpr uint32_t idesc = ptx::make_idesc(kDxfN, 128, 1, 1);
      const uint32_t lboA = (uint32_t)R * 16u;
      const uint64_t aDesc0 = ptx::smem_desc(sA_u, lboA, 128), wDesc0 = ptx::smem_desc(sW_u, kDxfN * 16, 128);
#ifdef TDM_WAIT_STATS
      long long issue_cycles = 0;  // time inside the MMA issue instruction (a full queue blocks it)
#endif
      int sa = 0;
      uint32_t pha = 0;
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      bool ok = TDM_TIMED_WAIT(2, wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_MMA));
      uint32_t j = 0;
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t >> 1) * MOUT;
        if (!tile_has_work(p, m0, MOUT)) continue;
        const uint32_t buf = j & 1u, use = j >> 1;
        if (!TDM_TIMED_WAIT(0, wait_or_flag(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * ACC_COLS;
        uint32_t accumulate = 0;
        for (int zt = 0; zt < 3 && ok; ++zt) {
          if (!TDM_TIMED_WAIT(1, wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
          ptx::tc_fence_after();
          // one thread issues every MMA: descriptors are advanced by adds, not rebuilt
          const uint64_t aStage = ptx::desc_advance(aDesc0, sa * a_stage);
#pragma unroll
          for (int dy = 0; dy < 3; ++dy) {
            const uint64_t aRow = ptx::desc_advance(aStage, (uint32_t)(dy * p.D) * 16u);
            const uint64_t wDesc = ptx::desc_advance(wDesc0, (uint32_t)(zt * 3 + dy) * kDxfBlock);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t bdesc = ptx::desc_advance(wDesc, (2 * kk) * kDxfN * 16);
#pragma unroll
              for (int i = 0; i < MSUB; ++i) {
                const uint64_t adesc = ptx::desc_advance(aRow, (2 * kk) * lboA + (uint32_t)(i * kDxfSub) * 16u);
#ifdef TDM_WAIT_STATS
                const long long c_issue = clock64();
#endif
                ptx::mma_f16(dbase + i * kDxfN, adesc, bdesc, idesc, accumulate);
#ifdef TDM_WAIT_STATS
                issue_cycles += clock64() - c_issue;
#endif
              }
              accumulate = 1;  // each sub-tile's first MMA (zt = dy = kk = 0) starts its accumulator
            }
          }
          ptx::mma_commit(emptyA + 8 * sa);
          if (++sa == kDxfNSA) { sa = 0; pha ^= 1; }
        }
        ptx::mma_commit(accFull + 8 * buf);
        ++j;
      }
      ptx::mma_commit(done);
      wait_or_flag(done, 0, p.err, DEV_TIMEOUT_MMA);
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[2], (unsigned long long)issue_cycles);
      atomicAdd(&g_wait_stats[6], (unsigned long long)(clock64() - t_loop0));
#endif
    }
  } else {
    // ---------------- epilogue (warps 2-5, TMEM lane quarter q = warp % 4) ----------------
    // Per tile: every quarter publishes the P_1 / P_2 values of its lanes 0
    // and 1 (both sub-tiles) in shared memory; barrier A (which also carries
    // the continue/stop vote and frees the output staging); outputs computed
    // into the staging area; barrier B; then one lane per output run issues
    // bulk shared -> global stores.  The epilogue threads themselves never
    // store to global memory, so no barrier waits for global stores.
    const uint32_t sO_u = ptx::smem_u32(sO);
    constexpr int CH = FP8_OUT ? 2 : 4;  // 16-byte output chunks per row of this half
#ifdef TDM_WAIT_STATS
    const long long t_epi0 = clock64();
#endif
    const int q = warp & 3;
    const int L = q * 32 + lane;  // TMEM lane = row within the 128-row sub-tile
    const int n0 = half * kDxfNt;
    bool issued = false;  // this lane has bulk stores in flight
    uint32_t j = 0;
    for (int64_t t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
      const int64_t m0 = (t >> 1) * MOUT;
      if (!tile_has_work(p, m0, MOUT)) continue;
      const uint32_t buf = j & 1u, use = j >> 1;
      const int got = __all_sync(
          0xffffffffu, TDM_TIMED_WAIT(5, wait_or_flag(accFull + 8 * buf, use & 1u, p.err, DEV_TIMEOUT_EPILOGUE)) ? 1 : 0);
      if (lane == 0) sVote[(j & 1u) * 4 + q] = got;
      float* xs = sX + (j & 1u) * (MSUB * 4 * 96);
      if (got) {
        ptx::tc_fence_after();
#pragma unroll
        for (int i = 0; i < MSUB; ++i) {
          const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_COLS + i * kDxfN;
#pragma unroll
          for (int c0 = 0; c0 < kDxfNt; c0 += 16) {
            uint32_t r1[16], r2[16];
            ptx::tmem_ld16_nowait(ta + kDxfNt + c0, r1);
            ptx::tmem_ld16_nowait(ta + 2 * kDxfNt + c0, r2);
            ptx::tmem_wait_ld();
            float* xw = xs + (i * 4 + q) * 96;
            if (lane == 0) {
#pragma unroll
              for (int e = 0; e < 16; ++e) { xw[c0 + e] = __uint_as_float(r1[e]); xw[32 + c0 + e] = __uint_as_float(r2[e]); }
            } else if (lane == 1) {
#pragma unroll
              for (int e = 0; e < 16; ++e) xw[64 + c0 + e] = __uint_as_float(r2[e]);
            }
          }
        }
      }
      if (issued) ptx::bulk_wait_read_all();  // the staging area is free again
      epi_bar();  // A
      const int* vote = sVote + (j & 1u) * 4;
      if (!(vote[0] && vote[1] && vote[2] && vote[3])) break;
#pragma unroll 1
      for (int i = 0; i < MSUB; ++i) {
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_COLS + i * kDxfN;
        const float* xn = xs + (i * 4 + ((q + 1) & 3)) * 96;  // next quarter (q = 3: rows >= 126 only)
#pragma unroll 1
        for (int c0 = 0; c0 < kDxfNt; c0 += 16) {
          uint32_t r0[16], r1[16], r2[16];
          ptx::tmem_ld16_nowait(ta + c0, r0);
          ptx::tmem_ld16_nowait(ta + kDxfNt + c0, r1);
          ptx::tmem_ld16_nowait(ta + 2 * kDxfNt + c0, r2);
          ptx::tmem_wait_ld();
          // neighbour-quarter values and biases: broadcast vector loads by
          // every lane and a select, so the shuffle loop has no branches
          float nb1[16], nb2a[16], nb2b[16], bi[16];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float4 u = reinterpret_cast<const float4*>(xn + c0)[k];
            const float4 w = reinterpret_cast<const float4*>(xn + 32 + c0)[k];
            const float4 z = reinterpret_cast<const float4*>(xn + 64 + c0)[k];
            const float4 c = __ldg(reinterpret_cast<const float4*>(p.bias + n0 + c0) + k);
            nb1[4 * k] = u.x; nb1[4 * k + 1] = u.y; nb1[4 * k + 2] = u.z; nb1[4 * k + 3] = u.w;
            nb2a[4 * k] = w.x; nb2a[4 * k + 1] = w.y; nb2a[4 * k + 2] = w.z; nb2a[4 * k + 3] = w.w;
            nb2b[4 * k] = z.x; nb2b[4 * k + 1] = z.y; nb2b[4 * k + 2] = z.z; nb2b[4 * k + 3] = z.w;
            bi[4 * k] = c.x; bi[4 * k + 1] = c.y; bi[4 * k + 2] = c.z; bi[4 * k + 3] = c.w;
          }
          const bool l31 = lane == 31, l30 = lane == 30;
          float v[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            float s1 = __shfl_down_sync(0xffffffffu, __uint_as_float(r1[e]), 1);
            float s2 = __shfl_down_sync(0xffffffffu, __uint_as_float(r2[e]), 2);
            s1 = l31 ? nb1[e] : s1;
            s2 = l31 ? nb2b[e] : (l30 ? nb2a[e] : s2);
            const float a = ((__uint_as_float(r0[e]) + s1) + s2) + bi[e];
            v[e] = p.relu ? fmaxf(a, 0.0f) : a;
          }
          // staging row: the lane's row, or in the x-pooled form the pair's (even
          // lanes store the max of the packed values of lanes L and L ^ 1; the
          // rounding is monotonic, so packing first gives the same bits)
          const bool stage = !XPOOL || (L & 1) == 0;
          const int SL = XPOOL ? (L >> 1) : L;
          // rows 126 and 127 of a sub-tile are staged too but never stored
          if (FP8_OUT) {
            uint4 o;
            o.x = pack_e4m3x4(v[0] * p.out_qinv, v[1] * p.out_qinv, v[2] * p.out_qinv, v[3] * p.out_qinv);
            o.y = pack_e4m3x4(v[4] * p.out_qinv, v[5] * p.out_qinv, v[6] * p.out_qinv, v[7] * p.out_qinv);
            o.z = pack_e4m3x4(v[8] * p.out_qinv, v[9] * p.out_qinv, v[10] * p.out_qinv, v[11] * p.out_qinv);
            o.w = pack_e4m3x4(v[12] * p.out_qinv, v[13] * p.out_qinv, v[14] * p.out_qinv, v[15] * p.out_qinv);
            if (XPOOL) {  // ReLU outputs: E4M3 bytes order like the values
              o.x = __vmaxu4(o.x, __shfl_xor_sync(0xffffffffu, o.x, 1));
              o.y = __vmaxu4(o.y, __shfl_xor_sync(0xffffffffu, o.y, 1));
              o.z = __vmaxu4(o.z, __shfl_xor_sync(0xffffffffu, o.z, 1));
              o.w = __vmaxu4(o.w, __shfl_xor_sync(0xffffffffu, o.w, 1));
            }
            if (stage) *reinterpret_cast<uint4*>(sO + ((i * 4 + c0 / 16) * 128 + SL) * 16) = o;
          } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              uint4 o;
              o.x = pack_bf16x2(v[8 * h + 0], v[8 * h + 1]);
              o.y = pack_bf16x2(v[8 * h + 2], v[8 * h + 3]);
              o.z = pack_bf16x2(v[8 * h + 4], v[8 * h + 5]);
              o.w = pack_bf16x2(v[8 * h + 6], v[8 * h + 7]);
              if (XPOOL) {
                uint32_t* w = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                  const uint32_t nb = __shfl_xor_sync(0xffffffffu, w[k], 1);
                  __nv_bfloat162 m = __hmax2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]),
                                             *reinterpret_cast<const __nv_bfloat162*>(&nb));
                  w[k] = *reinterpret_cast<uint32_t*>(&m);
                }
              }
              if (stage) *reinterpret_cast<uint4*>(sO + ((i * 4 + c0 / 8 + h) * 128 + SL) * 16) = o;
            }
          }
        }
      }
      ptx::tc_fence_before();
      ptx::fence_proxy_async_smem();  // staging writes visible to the bulk copies
      epi_bar();                      // B
      if (lane == 0) mbar_arrive(accEmpty + 8 * buf);
      // Output runs: sub-tile i spans rows [s, s + 126); every grid row
      // (b, z, y) of 28 inputs holds one run of up to 26 outputs.  Lane k of
      // quarter q = i handles the k-th grid row the sub-tile touches.
      if (q < MSUB) {
        const int64_t s0 = m0 + (int64_t)q * kDxfSub;
        const int64_t e0 = min(s0 + kDxfSub, p.rows);
        const bool rows32 = p.rows <= INT32_MAX;
        const int64_t y0 = row_div(s0, p.D, rows32);
        const int64_t yr = y0 + lane;  // grid row index (b*D + z)*D + y
        const int64_t ra = max(s0, yr * p.D), rb = min(e0, yr * p.D + p.Do);
        if (lane < 6 && ra < rb) {
          const int64_t bz = row_div(yr, p.D, rows32);  // b*D + z
          const int y = (int)(yr - bz * p.D);
          const int64_t b = row_div(bz, p.D, rows32);
          const int z = (int)(bz - b * p.D);
          if (y < p.Do && z < p.Do) {
            const int x = (int)(ra - yr * p.D);
            // x-pooled: x pairs (ra and rb are even), row pitch Do/2
            const int XO = XPOOL ? p.Do / 2 : p.Do;
            const int64_t pout = ((b * p.Do + z) * p.Do + y) * XO + (XPOOL ? x / 2 : x);
            const uint32_t len = (uint32_t)((rb - ra) / (XPOOL ? 2 : 1)) * 16u;
            const int srow = (int)(ra - s0) / (XPOOL ? 2 : 1);
#pragma unroll
            for (int c = 0; c < CH; ++c)
              ptx::bulk_s2g(p.out + (int64_t)(n0 / (FP8_OUT ? 16 : 8) + c) * p.out_cs + pout * 16,
                            sO_u + ((q * 4 + c) * 128 + srow) * 16, len);
            ptx::bulk_commit();
            issued = true;
          }
        }
      }
      ++j;
    }
    if (issued) ptx::bulk_wait_all();
#ifdef TDM_WAIT_STATS
    atomicAdd(&g_wait_stats[4], (unsigned long long)(clock64() - t_epi0));
#endif
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// conv2 on a CTA pair (cta_group::2).
//
// The dx-fused kernel above issues one N = 96 MMA (three dx taps x 32 output
// channels) per 128 rows and K step.  Such an MMA reads 7 KB of operands for
// 48 cycles of math, so it keeps the SM's shared-memory read port busy on its
// own (56 cycles alone), and the kernel's other shared-memory traffic (slab
// copies, output staging) stretches it further.  Here the two CTAs of a
// cluster share each MMA (tcgen05.mma.cta_group::2): M = 256 rows -- 128 from
// each CTA's slab -- by N = 192 columns, the three dx taps of all 64 output
// channels, whose weights are split between the CTAs exactly as the resident
// halves above (the leader's 110.6 KB give channels 0..31, the peer's
// 32..63).  Each SM still reads 7 KB per MMA, now for 96 cycles of math.
//
// A pair tile is 252 output rows of one z plane: the leader computes MMA rows
// [m0, m0 + 128) and stores outputs [m0, m0 + 126), the peer [m0 + 126, ...).
// Work units walk z through a column of such plane blocks, so consecutive
// tiles share two of their three z slabs (PairSched / pair_unit below).
// Roles:
//   warp 0, lane 0 (both CTAs): weights once, then its own half of each slab
//     by a tiled tensor copy (.cta_group::2) that completes on the leader's
//     barrier, one slab per tile;
//   warp 1, lane 0: the leader issues every MMA and commits with multicast to
//     both CTAs' barriers (stage free, accumulator full); the peer relays its
//     "weights landed" completion to the leader by a remote mbarrier arrive;
//   warps 2-17 (both CTAs): four epilogue sets of 16 output channels x four
//     TMEM lane quarters.  A warp reads its 48 accumulator columns (the three
//     dx taps of its channels), signals the leader's accumulator-empty barrier
//     at once (local, or a relaxed remote arrive: a release at cluster scope
//     held the warp ~1,000 cycles), then adds the row-shifted taps (lane
//     shuffles; the quarter boundary through shared memory), packs, and takes
//     the pool's x-pair max (lane L ^ 1), z-pair max (tiles z and z + 1 of a
//     unit go through the same warp) and, for y pairs within the CTA's rows,
//     the y-pair max (shared memory, one set barrier per odd tile), storing
//     each lane's 16-byte chunks straight to global memory.  Staging whole
//     tiles in shared memory for bulk stores cost the warp issuing them ~2,500
//     cycles a tile.
// TMEM: one pair allocation (issued together by warp 1 of both CTAs), two
// accumulator buffers of 192 columns.  Every mbarrier wait is bounded; both
// CTAs always reach the cluster barriers (no early exit), so a timeout in one
// CTA makes the other's waits run out too, and both free their TMEM.
// The sums are the kernel above's in the same order, so the outputs are the
// same bits.
// ---------------------------------------------------------------------------
constexpr int kD2EpiWarps = 16;                      // four sets of 16 channels x four lane quarters
constexpr int kD2Threads = 32 * (2 + kD2EpiWarps);
constexpr int kD2NSA = 4;                 // A slab stages per CTA (three per tile: one tile and a third in flight)
constexpr int kD2N = 2 * kDxfN;           // 192 accumulator columns per buffer
constexpr int kD2Out = 2 * kDxfSub;       // 252 output rows per pair tile
constexpr uint32_t kD2Xchg = 4u * 2u * 4u * 48u * 4u;  // [set][parity][quarter][P1 l0, P2 l0, P2 l1] x 16
constexpr int kD2Bars = 2 * kD2NSA + 7;
constexpr uint32_t kD2YStage = 64u * 4u * 32u;  // y-pair staging: [row / 2][set][32 B]
constexpr int64_t kPairMaxRows = INT32_MAX - (1 << 16);  // slab rows stay below 2^31

// Work units of the pair kernel: (patch b, block yb of 252 rows of a z plane,
// segment of zs output planes).  A unit's tiles walk z, so consecutive tiles
// share two of their three z slabs: a unit of nz tiles loads nz + 2 slabs.
// nyb blocks cover the rows of a plane that hold outputs (y < Do); nseg
// segments per column keep every pair busy on small batches.
struct PairSched {
  int nunits, nyb, nseg, zs;
};
struct PairUnit {
  int b, yb, z0, nz;
};
__device__ __forceinline__ PairUnit pair_unit(int u, const PairSched& ps, int Do) {
  const int col = u / ps.nseg, g = u - col * ps.nseg;
  PairUnit w;
  w.b = col / ps.nyb;
  w.yb = col - w.b * ps.nyb;
  w.z0 = g * ps.zs;
  w.nz = min(Do, w.z0 + ps.zs) - w.z0;
  return w;
}

__device__ __forceinline__ void epi_bar_set(int set) {
  // named barriers 1..4 (0 is __syncthreads), one per epilogue set of 4 warps
  asm volatile("bar.sync %0, 128;" ::"r"(set + 1) : "memory");
}

template <bool FP8_OUT, bool XPOOL, bool ZPOOL, bool YPOOL>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kD2Threads, 1) tc_conv_dxf2_kernel(const KParams p,
                                                                                          const __grid_constant__ CUtensorMap tmA,
                                                                                          const PairSched ps) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t TMEM_COLS = 512;
  const int R = p.R;
  const uint32_t a_stage = 16u * 8u * (uint32_t)R;
  uint8_t* sW = smem;
  uint8_t* sA = smem + kDxfWBytes;
  float* sX = reinterpret_cast<float*>(sA + kD2NSA * a_stage);
  uint4* sY = reinterpret_cast<uint4*>(reinterpret_cast<uint8_t*>(sX) + kD2Xchg);  // y-pair staging
  float* sBias = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(sY) + kD2YStage);  // the layer's 64 biases
  int* sVote = reinterpret_cast<int*>(sBias + 64);  // [set][parity][quarter]
  uint64_t* bars = reinterpret_cast<uint64_t*>(sVote + 32);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + kD2Bars);

  const uint32_t rank = ptx::cluster_rank();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // a CTA that starts with the error word raised skips its loops but still
  // meets its peer at both cluster barriers
  const bool skip = !__syncthreads_and(aborted(p.err) ? 0 : 1);

  // fullA is used in the leader only (both CTAs' slab copies complete on it)
  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * kD2NSA;
  const uint32_t wfull = emptyA + 8 * kD2NSA, peerW = wfull + 8, accFull = peerW + 8, accEmpty = accFull + 16,
                 done = accEmpty + 16;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kD2NSA; ++i) {
      ptx::mbar_init(fullA + 8 * i, 1);
      ptx::mbar_init(emptyA + 8 * i, 1);
    }
    ptx::mbar_init(wfull, 1);
    ptx::mbar_init(peerW, 1);
    for (int i = 0; i < 2; ++i) {
      ptx::mbar_init(accFull + 8 * i, 1);
      ptx::mbar_init(accEmpty + 8 * i, 2 * kD2EpiWarps);  // every epilogue warp of both CTAs
    }
    ptx::mbar_init(done, 1);
    ptx::fence_barrier_init();
    ptx::fence_proxy_async_smem();
  }
  if (warp == 1) {
    ptx::tmem_alloc2(ptx::smem_u32(tmem_holder), TMEM_COLS);
    ptx::tmem_relinquish2();
  }
  if (threadIdx.x >= 64 && threadIdx.x < 128) sBias[threadIdx.x - 64] = p.bias[threadIdx.x - 64];
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // both CTAs' barriers exist before any remote arrive or multicast commit
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t sA_u = ptx::smem_u32(sA), sW_u = ptx::smem_u32(sW);
  const int64_t plane = (int64_t)p.D * p.D;
  const int64_t pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;

  if (warp == 0) {
    if (lane == 0 && !skip) {
      // ---------------- producer: this CTA's weight half once, then its A slabs ----------------
      ptx::mbar_arrive_expect_tx(wfull, kDxfWBytes);
      for (int b = 0; b < 9; ++b)
        ptx::bulk_g2s(sW_u + b * kDxfBlock, p.wpk + (size_t)rank * kDxfWBytes + (size_t)b * kDxfBlock, kDxfBlock,
                      wfull);
      // Slabs: one tiled copy of [8 chunks][R rows][16 B] per stage.  Both
      // CTAs' copies complete on the leader's fullA (the leader expects both
      // halves' bytes), so the MMA issuer waits on one local barrier per stage.
      // The peer loads stage s of use k only after the MMAs of use k - 1 freed
      // it (emptyA, multicast), i.e. after the leader's fullA left that phase.
      // Slab n of this CTA (counted over all its units) goes to stage
      // n % NSA; a unit of nz tiles loads its nz + 2 z slabs once.
      const uint32_t fullA_lead = ptx::mapa_shared(fullA, 0);
      int armedA[kD2NSA];
      for (int i = 0; i < kD2NSA; ++i) armedA[i] = -1;
      bool ok = true;
      uint32_t n = 0;
      for (int u = (int)pair; u < ps.nunits && ok; u += (int)npairs) {
        const PairUnit w = pair_unit(u, ps, p.Do);
        const int64_t base = w.b * (int64_t)plane * p.D + w.yb * kD2Out + (int64_t)rank * kDxfSub + (int64_t)w.z0 * plane;
        for (int k = 0; k < w.nz + 2; ++k, ++n) {
          const uint32_t sa = n % kD2NSA, pha = (n / kD2NSA) & 1u;
          if (!TDM_TIMED_WAIT(3, wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
          if (rank == 0) ptx::mbar_arrive_expect_tx(fullA + 8 * sa, 2 * a_stage);
          armedA[sa] = (int)pha;
          ptx::tma_load_3d_pair(sA_u + sa * a_stage, &tmA, 0, (int)((base + k * plane) >> 1), 0, fullA_lead + 8 * sa);
        }
      }
      if (rank == 0) {
        // the leader's fullA phases cover both CTAs' copies
        for (int i = 0; i < kD2NSA; ++i)
          if (armedA[i] >= 0) wait_or_flag(fullA + 8 * i, (uint32_t)armedA[i], p.err, DEV_TIMEOUT_PRODUCER);
      } else if (aborted(p.err)) {
        // the peer cannot see its copies complete; after an abort it gives
        // any still in flight 200 us (one lands within a few microseconds)
        const uint64_t t0 = ptx::globaltimer_ns();
        while (ptx::globaltimer_ns() - t0 < 200000ull) __nanosleep(1000);
      }
      wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_PRODUCER);
    }
  } else if (warp == 1) {
    if (lane == 0 && !skip && rank == 1) {
      // ---------------- peer: relay its weight copy's completion to the leader ----------------
      if (wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_PRODUCER)) ptx::mbar_arrive_remote(peerW, 0);
    } else if (lane == 0 && !skip && rank == 0) {
      // ---------------- leader: the pair's MMA issuer ----------------
      constexpr uint32_t idesc = ptx::make_idesc(kD2N, 256, 1, 1);
      const uint32_t lboA = (uint32_t)R * 16u;
      const uint64_t aDesc0 = ptx::smem_desc(sA_u, lboA, 128), wDesc0 = ptx::smem_desc(sW_u, kDxfN * 16, 128);
      bool ok = wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_MMA) &&
                wait_or_flag_cluster(peerW, 0, p.err, DEV_TIMEOUT_MMA);
      uint32_t n = 0, j = 0;
#ifdef TDM_WAIT_STATS
      const long long t_loop0 = clock64();
#endif
      for (int u = (int)pair; u < ps.nunits && ok; u += (int)npairs) {
        const PairUnit w = pair_unit(u, ps, p.Do);
        for (int zi = 0; zi < w.nz && ok; ++zi) {
        const uint32_t buf = j & 1u, use = j >> 1;
        if (!TDM_TIMED_WAIT(0, wait_or_flag_cluster(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * kD2N;
        uint32_t accumulate = 0;
        for (int zt = 0; zt < 3 && ok; ++zt) {
          // tile zi reads slabs zi, zi + 1, zi + 2 of the unit; each slab is
          // waited for at its first use (the unit's first tile, else zt = 2)
          const uint32_t sn = n + zi + zt, sa = sn % kD2NSA, pha = (sn / kD2NSA) & 1u;
          if (zi == 0 || zt == 2) {
            if (!TDM_TIMED_WAIT(1, wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA))) {
              ok = false;
              break;
            }
            ptx::tc_fence_after();
          }
          const uint64_t aStage = ptx::desc_advance(aDesc0, sa * a_stage);
#pragma unroll
          for (int dy = 0; dy < 3; ++dy) {
            const uint64_t aRow = ptx::desc_advance(aStage, (uint32_t)(dy * p.D) * 16u);
            const uint64_t wDesc = ptx::desc_advance(wDesc0, (uint32_t)(zt * 3 + dy) * kDxfBlock);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              ptx::mma2_f16(dbase, ptx::desc_advance(aRow, (2 * kk) * lboA),
                            ptx::desc_advance(wDesc, (2 * kk) * kDxfN * 16), idesc, accumulate);
              accumulate = 1;
            }
          }
          // a slab's last use: zt = 0, or any zt of the unit's last tile
          if (zt == 0 || zi == w.nz - 1) ptx::mma2_commit_both(emptyA + 8 * sa);
        }
        if (!ok) break;
        ptx::mma2_commit_both(accFull + 8 * buf);
        ++j;
        }
        n += w.nz + 2;
      }
#ifdef TDM_WAIT_STATS
      atomicAdd(&g_wait_stats[6], (unsigned long long)(clock64() - t_loop0));
#endif
      ptx::mma2_commit_both(done);
      wait_or_flag(done, 0, p.err, DEV_TIMEOUT_MMA);
    }
  } else if (!skip) {
    // ---------------- epilogue: set = 16 output channels, TMEM lane quarter q = warp % 4 ----------------
    const int set = (warp - 2) >> 2;  // 0..3
    const int q = warp & 3;
    const int L = q * 32 + lane;  // TMEM lane = row within the CTA's 128 rows
    const int n0 = set * 16;      // first output channel of this set
    // this set's columns: channel half set / 2 (the 96 columns of its dx taps),
    // 16 channels at (set % 2) * 16 within each tap's 32
    const uint32_t col0 = (uint32_t)((set >> 1) * kDxfN + (set & 1) * 16);
    static_assert(!ZPOOL || XPOOL, "the z-pair max comes with the x-pair max");
    static_assert(!YPOOL || ZPOOL, "the y-pair max comes with the x- and z-pair max");
    const int Do = p.Do, XO = XPOOL ? p.Do / 2 : p.Do, ZO = ZPOOL ? p.Do / 2 : p.Do;
    uint8_t* const outp = p.out + (int64_t)(n0 / (FP8_OUT ? 16 : 8)) * p.out_cs;
    uint8_t* const outp2 = YPOOL ? p.out2 + (int64_t)(n0 / (FP8_OUT ? 16 : 8)) * p.out_cs : nullptr;
    uint32_t j = 0;
    bool stop = false;
    // z-pooled: units start on even z with an even number of tiles, and the
    // same warp drains tiles z and z + 1 one after the other, so it keeps the
    // even tile's packed output here and stores the max with the odd one
    uint4 zkeep[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    for (int u = (int)pair; u < ps.nunits && !stop; u += (int)npairs) {
      const PairUnit w = pair_unit(u, ps, Do);
      // this lane's row within a z plane (the same for every tile of the
      // unit) and its output offset at z = 0, or -1 (rows L < 126 of this
      // CTA's half, x, y < Do; x-pooled: the even rows hold the pair maxima)
      const int pp = w.yb * kD2Out + (int)rank * kDxfSub + L, y = pp / p.D, x = pp - y * p.D;
      const bool lane_ok = L < kDxfSub && x < Do && y < Do && (!XPOOL || (x & 1) == 0);
      const int pbase = ((w.b * ZO + (ZPOOL ? w.z0 / 2 : w.z0)) * Do + y) * XO + (XPOOL ? x / 2 : x);
      // y-pooled: the rows of y and y + 1 (y even) at the same x are D apart;
      // when both lie in this CTA's 126 rows they meet in shared memory and the
      // even one stores the pooled row, otherwise (ycross) both go out x- and
      // z-pooled and the pool pass takes their max
      const bool ycross = YPOOL && ((y & 1) ? L < p.D : L + p.D >= kDxfSub);
      const int fbase = YPOOL ? ((w.b * ZO + w.z0 / 2) * (Do / 2) + y / 2) * XO + x / 2 : 0;
      for (int zi = 0; zi < w.nz; ++zi) {
      const int pout = lane_ok ? pbase + (ZPOOL ? zi / 2 : zi) * Do * XO : -1;
      const bool zstore = !ZPOOL || (zi & 1);  // z-pooled: the odd tile of each z pair stores
      const int pfin = fbase + (zi / 2) * (Do / 2) * XO;  // y-pooled output row (when pout >= 0)
      const uint32_t buf = j & 1u, use = j >> 1;
      const int got = __all_sync(0xffffffffu, wait_or_flag(accFull + 8 * buf, use & 1u, p.err, DEV_TIMEOUT_EPILOGUE) ? 1 : 0);
      int* vote = sVote + (set * 2 + (j & 1u)) * 4;
      if (lane == 0) vote[q] = got;
      // The exchange: the previous quarter's lanes 30 and 31 need this
      // quarter's lane 0 (P1, P2) and lane 1 (P2) values (rows +1 and +2 cross
      // the 32-lane boundary), published before barrier A.  The buffers
      // alternate by tile parity: tile j + 2 writes them only after every warp
      // of the set has passed barrier A of tile j + 1, i.e. finished reading
      // tile j's.
      float* xs = sX + (set * 2 + (j & 1u)) * (4 * 48);
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + buf * kD2N + col0;
      uint32_t r0v[16], r1v[16], r2v[16];
      if (got) {
        ptx::tc_fence_after();
        // all three loads in flight before one wait
        ptx::tmem_ld16_nowait(ta, r0v);
        ptx::tmem_ld16_nowait(ta + kDxfNt, r1v);
        ptx::tmem_ld16_nowait(ta + 2 * kDxfNt, r2v);
        ptx::tmem_wait_ld();
        // this warp has read all it needs of the buffer: hand it back to the
        // MMA issuer now, before the exchange, the arithmetic and the stores
        ptx::tc_fence_before();
        if (lane == 0) {
          if (rank == 0) mbar_arrive(accEmpty + 8 * buf);
          else ptx::mbar_arrive_remote_relaxed(accEmpty + 8 * buf, 0);
        }
        uint4* xw = reinterpret_cast<uint4*>(xs + q * 48);
        if (lane == 0) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            xw[k] = make_uint4(r1v[4 * k], r1v[4 * k + 1], r1v[4 * k + 2], r1v[4 * k + 3]);
            xw[4 + k] = make_uint4(r2v[4 * k], r2v[4 * k + 1], r2v[4 * k + 2], r2v[4 * k + 3]);
          }
        } else if (lane == 1) {
#pragma unroll
          for (int k = 0; k < 4; ++k) xw[8 + k] = make_uint4(r2v[4 * k], r2v[4 * k + 1], r2v[4 * k + 2], r2v[4 * k + 3]);
        }
      }
      epi_bar_set(set);  // A
      if (!(vote[0] && vote[1] && vote[2] && vote[3])) {
        stop = true;
        break;
      }
      const float* xn = xs + ((q + 1) & 3) * 48;  // next quarter (q = 3: rows >= 126 only)
      const bool l31 = lane == 31, l30 = lane == 30;
      // the 16 outputs, packed four channels at a time as they are made
      // (E4M3: one word per four, BF16: two), which keeps few registers live
      uint32_t pk[FP8_OUT ? 4 : 8];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        // neighbour-quarter values and biases: broadcast shared-memory loads
        const float4 u = reinterpret_cast<const float4*>(xn)[k];
        const float4 w = reinterpret_cast<const float4*>(xn + 16)[k];
        const float4 zz = reinterpret_cast<const float4*>(xn + 32)[k];
        const float4 c = reinterpret_cast<const float4*>(sBias + n0)[k];
        const float nb1[4] = {u.x, u.y, u.z, u.w}, nb2a[4] = {w.x, w.y, w.z, w.w};
        const float nb2b[4] = {zz.x, zz.y, zz.z, zz.w}, bi[4] = {c.x, c.y, c.z, c.w};
        float v[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int e = 4 * k + i;
          float s1 = __shfl_down_sync(0xffffffffu, __uint_as_float(r1v[e]), 1);
          float s2 = __shfl_down_sync(0xffffffffu, __uint_as_float(r2v[e]), 2);
          s1 = l31 ? nb1[i] : s1;
          s2 = l31 ? nb2b[i] : (l30 ? nb2a[i] : s2);
          const float a = ((__uint_as_float(r0v[e]) + s1) + s2) + bi[i];
          v[i] = p.relu ? fmaxf(a, 0.0f) : a;
        }
        if (FP8_OUT) {
          pk[k] = pack_e4m3x4(v[0] * p.out_qinv, v[1] * p.out_qinv, v[2] * p.out_qinv, v[3] * p.out_qinv);
        } else {
          pk[2 * k] = pack_bf16x2(v[0], v[1]);
          pk[2 * k + 1] = pack_bf16x2(v[2], v[3]);
        }
      }
      // stores straight from registers: chunk-planar output, 16 B per row
      // and chunk; a warp's even lanes write consecutive pooled rows
      if (FP8_OUT) {
        uint4 o = make_uint4(pk[0], pk[1], pk[2], pk[3 % (FP8_OUT ? 4 : 8)]);
        if (XPOOL) {
          o.x = __vmaxu4(o.x, __shfl_xor_sync(0xffffffffu, o.x, 1));
          o.y = __vmaxu4(o.y, __shfl_xor_sync(0xffffffffu, o.y, 1));
          o.z = __vmaxu4(o.z, __shfl_xor_sync(0xffffffffu, o.z, 1));
          o.w = __vmaxu4(o.w, __shfl_xor_sync(0xffffffffu, o.w, 1));
        }
        if (ZPOOL) {
          if (zi & 1) {
            o.x = __vmaxu4(o.x, zkeep[0].x);
            o.y = __vmaxu4(o.y, zkeep[0].y);
            o.z = __vmaxu4(o.z, zkeep[0].z);
            o.w = __vmaxu4(o.w, zkeep[0].w);
          } else {
            zkeep[0] = o;
          }
        }
        if (!YPOOL && zstore && pout >= 0) *reinterpret_cast<uint4*>(outp + (int64_t)pout * 16) = o;
        if (YPOOL && zstore) {
          if (pout >= 0) {
            if (ycross) *reinterpret_cast<uint4*>(outp + (int64_t)pout * 16) = o;
            else sY[(L >> 1) * 4 + set] = o;
          }
          epi_bar_set(set);  // every warp of the set, every odd tile
          if (pout >= 0 && !ycross && (y & 1) == 0) {
            const uint4 m = sY[((L + p.D) >> 1) * 4 + set];
            o.x = __vmaxu4(o.x, m.x);
            o.y = __vmaxu4(o.y, m.y);
            o.z = __vmaxu4(o.z, m.z);
            o.w = __vmaxu4(o.w, m.w);
            *reinterpret_cast<uint4*>(outp2 + (int64_t)pfin * 16) = o;
          }
        }
      } else {
        uint4 ov[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint4 o = make_uint4(pk[(4 * h) % (FP8_OUT ? 4 : 8)], pk[(4 * h + 1) % (FP8_OUT ? 4 : 8)],
                               pk[(4 * h + 2) % (FP8_OUT ? 4 : 8)], pk[(4 * h + 3) % (FP8_OUT ? 4 : 8)]);
          if (XPOOL) {
            uint32_t* w = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const uint32_t nb = __shfl_xor_sync(0xffffffffu, w[k], 1);
              __nv_bfloat162 m = __hmax2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]),
                                         *reinterpret_cast<const __nv_bfloat162*>(&nb));
              w[k] = *reinterpret_cast<uint32_t*>(&m);
            }
          }
          if (ZPOOL) {
            if (zi & 1) {
              uint32_t* w = reinterpret_cast<uint32_t*>(&o);
              const uint32_t* kv = reinterpret_cast<const uint32_t*>(&zkeep[h]);
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                __nv_bfloat162 m = __hmax2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]),
                                           *reinterpret_cast<const __nv_bfloat162*>(&kv[k]));
                w[k] = *reinterpret_cast<uint32_t*>(&m);
              }
            } else {
              zkeep[h] = o;
            }
          }
          ov[h] = o;
          if (!YPOOL && zstore && pout >= 0) *reinterpret_cast<uint4*>(outp + h * p.out_cs + (int64_t)pout * 16) = o;
        }
        if (YPOOL && zstore) {
          // a row whose y pair shares the CTA half goes to shared memory, the
          // others out x- and z-pooled; the even row of a pair stores the max
          if (pout >= 0) {
            if (ycross) {
              *reinterpret_cast<uint4*>(outp + (int64_t)pout * 16) = ov[0];
              *reinterpret_cast<uint4*>(outp + p.out_cs + (int64_t)pout * 16) = ov[1];
            } else {
              sY[((L >> 1) * 4 + set) * 2] = ov[0];
              sY[((L >> 1) * 4 + set) * 2 + 1] = ov[1];
            }
          }
          epi_bar_set(set);  // every warp of the set, every odd tile
          if (pout >= 0 && !ycross && (y & 1) == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint4 m = sY[(((L + p.D) >> 1) * 4 + set) * 2 + h];
              uint32_t* wv = reinterpret_cast<uint32_t*>(&ov[h]);
              const uint32_t* mv = reinterpret_cast<const uint32_t*>(&m);
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                __nv_bfloat162 mx = __hmax2(*reinterpret_cast<const __nv_bfloat162*>(&wv[k]),
                                            *reinterpret_cast<const __nv_bfloat162*>(&mv[k]));
                wv[k] = *reinterpret_cast<uint32_t*>(&mx);
              }
              *reinterpret_cast<uint4*>(outp2 + h * p.out_cs + (int64_t)pfin * 16) = ov[h];
            }
          }
        }
      }
      ++j;
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::cluster_sync();  // the pair's MMAs are done and both CTAs have read their accumulators
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc2(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// conv1 with the im2col operand built in shared memory.  conv1 (1 input
// channel, 27 taps) is a GEMM over the 28^3 output positions of each patch
// with K = 27 taps padded to 32 and N = 64.  Instead of writing that operand
// to HBM (1.4 MB per patch) and reading it back, four producer warps gather
// the 27 FP32 taps of each row straight from the patch, convert them to BF16
// and store the row into the K-major stage ([chunk][row][16 B]); the MMA and
// epilogue roles are those of the generic kernel (N = 64, four 128-row
// sub-tiles, two TMEM buffers), and the 4 KB of weights stay resident.
// ---------------------------------------------------------------------------
constexpr int kC1Prod = 4;                            // producer warps
constexpr int kC1Threads = 32 * (kC1Prod + 1 + 4);    // + MMA warp + 4 epilogue warps
constexpr int kC1Rows = 512;                          // rows per tile (4 sub-tiles)
constexpr int kC1NSA = 3;                             // A stages
constexpr uint32_t kC1Stage = 4u * kC1Rows * 16u;     // 32 KB
constexpr uint32_t kC1W = 4u * 64u * 16u;             // weights: 4 chunks x 64 rows x 16 B
constexpr int kC1TilesPerPatch = (21952 + kC1Rows - 1) / kC1Rows;  // 43
constexpr int kC1PlaneSpan = 4 * 900;                 // floats: the <= 4 input z planes of a tile

struct C1Params {
  const float* patches;
  int64_t rows;  // B * 28^3
  const uint8_t* wpk;
  const float* bias;
  uint8_t* out;
  int64_t out_cs;
  int64_t tiles;
  int* err;
};

__global__ void __launch_bounds__(kC1Threads, 1) tc_conv1_kernel(const C1Params p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t ACC = 4 * 64;  // one buffer: 4 sub-tiles x N 64
  uint8_t* sW = smem;
  uint8_t* sA = smem + kC1W;
  float* sP = reinterpret_cast<float*>(sA + kC1NSA * kC1Stage);  // [2][kC1PlaneSpan] input planes
  uint64_t* bars = reinterpret_cast<uint64_t*>(sP + 2 * kC1PlaneSpan);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * kC1NSA + 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!__syncthreads_and(aborted(p.err) ? 0 : 1)) return;
  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * kC1NSA;
  const uint32_t wfull = emptyA + 8 * kC1NSA, accFull = wfull + 8, accEmpty = accFull + 16, done = accEmpty + 16,
                 fullP = done + 8;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kC1NSA; ++i) {
      ptx::mbar_init(fullA + 8 * i, 32 * kC1Prod);  // every producer thread arrives
      ptx::mbar_init(emptyA + 8 * i, 1);
    }
    ptx::mbar_init(wfull, 1);
    for (int i = 0; i < 2; ++i) { ptx::mbar_init(accFull + 8 * i, 1); ptx::mbar_init(accEmpty + 8 * i, 4); }
    ptx::mbar_init(done, 1);
    for (int i = 0; i < 2; ++i) ptx::mbar_init(fullP + 8 * i, 1);
    ptx::fence_barrier_init();
    ptx::fence_proxy_async_smem();
  }
  if (warp == kC1Prod) {
    ptx::tmem_alloc(ptx::smem_u32(tmem_holder), 512);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t sA_u = ptx::smem_u32(sA), sW_u = ptx::smem_u32(sW);

  if (warp < kC1Prod) {
    // ---------------- producers: im2col rows into the stages ----------------
    // A tile is 512 rows of one patch (43 tiles per patch, the last one 448
    // rows).  Its rows need at most four consecutive z planes of the 30^3
    // patch (14.4 KB): thread 0 copies them into shared memory one tile ahead
    // (two buffers), and the 27 taps of each row are read from there.
    const int pt = threadIdx.x;  // 0 .. 127
    const uint32_t sP_u = ptx::smem_u32(sP);
    if (pt == 0) {
      ptx::mbar_arrive_expect_tx(wfull, kC1W);
      ptx::bulk_g2s(sW_u, p.wpk, kC1W, wfull);
    }
    auto planes_copy = [&](int64_t t, int buf) {  // thread 0: the tile's input planes
      const int64_t b = t / kC1TilesPerPatch;
      const int r0 = (int)(t - b * kC1TilesPerPatch) * kC1Rows, r1 = min(21952, r0 + kC1Rows);
      const int zlo = r0 / 784, np = (r1 - 1) / 784 - zlo + 3;
      const uint32_t bytes = (uint32_t)np * 900u * 4u;
      ptx::mbar_arrive_expect_tx(fullP + 8 * buf, bytes);
      ptx::bulk_g2s(sP_u + (uint32_t)buf * kC1PlaneSpan * 4u, p.patches + b * 27000 + (int64_t)zlo * 900, bytes,
                    fullP + 8 * buf);
    };
    int sa = 0;
    uint32_t pha = 0;
    bool ok = true;
    int64_t issued = -1, waited = -1;  // thread 0: local tile index of the last plane copy issued / waited for
    constexpr int kRowsPerThread = kC1Rows / (32 * kC1Prod);
    if (pt == 0 && (int64_t)blockIdx.x < p.tiles) {
      planes_copy(blockIdx.x, 0);
      issued = 0;
    }
    uint32_t k = 0;
    for (int64_t t = blockIdx.x; t < p.tiles && ok; t += gridDim.x, ++k) {
      const int buf = (int)(k & 1u);
      if (pt == 0 && t + gridDim.x < p.tiles) {
        planes_copy(t + gridDim.x, buf ^ 1);
        issued = k + 1;
      }
      const int64_t b = t / kC1TilesPerPatch;
      const int r0 = (int)(t - b * kC1TilesPerPatch) * kC1Rows, nrows = min(kC1Rows, 21952 - r0);
      const int zlo = r0 / 784;
      const bool okP = wait_or_flag(fullP + 8 * buf, (k >> 1) & 1u, p.err, DEV_TIMEOUT_PRODUCER);
      if (pt == 0 && okP) waited = k;
      const float* sp = sP + buf * kC1PlaneSpan;
      float v[kRowsPerThread][27];
#pragma unroll
      for (int kr = 0; kr < kRowsPerThread; ++kr) {
        // rows past the tile's end read a valid row and store zeros
        const int r = r0 + min(pt + 32 * kC1Prod * kr, nrows - 1);
        const int z = r / 784 - zlo, y = (r / 28) % 28, x = r % 28;
        const float* src = sp + z * 900 + y * 30 + x;
#pragma unroll
        for (int tp = 0; tp < 27; ++tp) v[kr][tp] = src[(tp / 9) * 900 + ((tp / 3) % 3) * 30 + (tp % 3)];
      }
      const bool okA = wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER);
      // Every producer has read this plane buffer (thread 0 refills it next
      // tile), and all 128 learn together whether both waits succeeded, so
      // they leave the loop together and this barrier is always met.
      int all;
      asm volatile(
          "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.and.pred q, 1, %2, p;\n\t"
          "selp.s32 %0, 1, 0, q;\n\t}"
          : "=r"(all)
          : "r"((okP && okA) ? 1 : 0), "r"(32 * kC1Prod)
          : "memory");
      if (!all) {
        ok = false;
        break;
      }
      uint8_t* st = sA + sa * kC1Stage;
#pragma unroll
      for (int kr = 0; kr < kRowsPerThread; ++kr) {
        const int r = pt + 32 * kC1Prod * kr;
        const float keep = r < nrows ? 1.0f : 0.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float f[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) f[e] = 8 * j + e < 27 ? v[kr][8 * j + e] * keep : 0.0f;
          uint4 o;
          o.x = pack_bf16x2(f[0], f[1]);
          o.y = pack_bf16x2(f[2], f[3]);
          o.z = pack_bf16x2(f[4], f[5]);
          o.w = pack_bf16x2(f[6], f[7]);
          *reinterpret_cast<uint4*>(st + ((size_t)j * kC1Rows + r) * 16) = o;
        }
      }
      ptx::fence_proxy_async_smem();  // generic-proxy stores visible to the tensor core
      mbar_arrive(fullA + 8 * sa);
      if (++sa == kC1NSA) { sa = 0; pha ^= 1; }
    }
    if (pt == 0) {
      if (issued > waited) {
        // a plane copy issued for a tile the loop did not reach: let it land
        // (bounded); after an abort give any copy in flight 200 us
        const uint32_t kk = (uint32_t)issued;
        if (!wait_or_flag(fullP + 8 * (kk & 1u), (kk >> 1) & 1u, p.err, DEV_TIMEOUT_PRODUCER)) {
          const uint64_t t0 = ptx::globaltimer_ns();
          while (ptx::globaltimer_ns() - t0 < 200000ull) __nanosleep(1000);
        }
      }
      wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_PRODUCER);
    }
  } else if (warp == kC1Prod) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      constexpr uint32_t idesc = ptx::make_idesc(64, 128, 1, 1);
      constexpr uint32_t lboA = kC1Rows * 16u;
      const uint64_t aDesc0 = ptx::smem_desc(sA_u, lboA, 128), wDesc0 = ptx::smem_desc(sW_u, 64 * 16, 128);
      int sa = 0;
      uint32_t pha = 0;
      bool ok = wait_or_flag(wfull, 0, p.err, DEV_TIMEOUT_MMA);
      uint32_t j = 0;
      for (int64_t t = blockIdx.x; t < p.tiles && ok; t += gridDim.x) {
        const uint32_t buf = j & 1u, use = j >> 1;
        if (!wait_or_flag(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA)) { ok = false; break; }
        if (!wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA)) { ok = false; break; }
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * ACC;
        const uint64_t aStage = ptx::desc_advance(aDesc0, sa * kC1Stage);
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
          const uint64_t bdesc = ptx::desc_advance(wDesc0, (2 * kk) * 64 * 16);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const uint64_t adesc = ptx::desc_advance(aStage, (2 * kk) * lboA + (uint32_t)(i * 128) * 16u);
            ptx::mma_f16(dbase + i * 64, adesc, bdesc, idesc, kk > 0 ? 1u : 0u);
          }
        }
        ptx::mma_commit(emptyA + 8 * sa);
        if (++sa == kC1NSA) { sa = 0; pha ^= 1; }
        ptx::mma_commit(accFull + 8 * buf);
        ++j;
      }
      ptx::mma_commit(done);
      wait_or_flag(done, 0, p.err, DEV_TIMEOUT_MMA);
    }
  } else {
    // ---------------- epilogue: bias, ReLU, BF16 rows (conv2's chunk-planar input) ----------------
    const int q = warp & 3;
    float bias[64];  // loaded once: every row of every tile adds the same 64 biases
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float b16[16];
      load16(p.bias + 16 * k, b16);
#pragma unroll
      for (int e = 0; e < 16; ++e) bias[16 * k + e] = b16[e];
    }
    uint32_t j = 0;
    for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x) {
      const uint32_t buf = j & 1u, use = j >> 1;
      const bool have =
          __all_sync(0xffffffffu, wait_or_flag(accFull + 8 * buf, use & 1u, p.err, DEV_TIMEOUT_EPILOGUE) ? 1 : 0) != 0;
      if (!have) break;
      ptx::tc_fence_after();
#pragma unroll 1
      for (int i = 0; i < 4; ++i) {
        const int64_t b = t / kC1TilesPerPatch;
        const int rp = (int)(t - b * kC1TilesPerPatch) * kC1Rows + i * 128 + q * 32 + lane;  // row in the patch
        const bool valid = rp < 21952;
        const int64_t row = b * 21952 + rp;
        uint32_t r[4][16];  // the row's 64 accumulators: four loads, one wait
#pragma unroll
        for (int k = 0; k < 4; ++k)
          ptx::tmem_ld16_nowait(tmem + ((uint32_t)(q * 32) << 16) + buf * ACC + (uint32_t)(i * 64 + 16 * k), r[k]);
        ptx::tmem_wait_ld();
        if (!valid) continue;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          float f[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) f[e] = fmaxf(__uint_as_float(r[c / 2][8 * (c % 2) + e]) + bias[8 * c + e], 0.0f);
          uint4 o;
          o.x = pack_bf16x2(f[0], f[1]);
          o.y = pack_bf16x2(f[2], f[3]);
          o.z = pack_bf16x2(f[4], f[5]);
          o.w = pack_bf16x2(f[6], f[7]);
          *reinterpret_cast<uint4*>(p.out + (int64_t)c * p.out_cs + row * 16) = o;
        }
      }
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(accEmpty + 8 * buf);
      ++j;
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == kC1Prod) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

// A slab rows per CTA of the pair form: its 128 MMA rows shifted by up to 2 D
int pair_slab_rows(const TcLayer& L) { return 128 + 2 * L.D; }

int slab_rows(const TcLayer& L) {
  if (L.dxf) return (L.msub - 1) * kDxfSub + 128 + 2 * L.D;  // exact: the stages must fit beside the weights
  int r = L.msub * 128 + (L.nyx > 1 ? 2 * L.D + 2 : 0);
  return (r + 7) & ~7;
}

int chunks_per_group(const TcLayer& L) {
  // a K group is 128 bytes per row: 8 chunks, unless the layer has fewer channels
  int elem = L.fp8_in ? 16 : 8;  // channels per 16-byte chunk
  int chunks = L.cin / elem;
  return chunks < 8 ? chunks : 8;
}

size_t a_stage_bytes(const TcLayer& L) { return (size_t)16 * chunks_per_group(L) * slab_rows(L); }

// gathered-row form: one (tap, K group) of msub*128 rows per A stage
size_t gather_stage_bytes(const TcLayer& L) {
  return (size_t)16 * chunks_per_group(L) * (L.msub * 128 + (L.xrun ? 8 : 0));
}
int gather_stages(const TcLayer& L) { return L.xrun ? kXNSA : kGNSA; }
// weights-as-A epilogue: 8 warps x 16 rows x 32 channels of BF16, 16-byte aligned
constexpr size_t kWtStage = 8 * 16 * 32 * 2 + 16;

// A stages of the grid-form kernel: a GEMM's stage (one K group of msub*128
// rows) feeds a single weight stage, so as many as fit (up to MAX_NSA, leaving
// room for four weight stages) stay in flight
int grid_a_stages(const TcLayer& L) {
  if (!(L.nz == 1 && L.nyx == 1)) return NSA;
  const size_t left = kSmemLimit - kSmemReserve - 4 * (size_t)L.nt * 128;
  const int n = (int)(left / a_stage_bytes(L));
  return n < NSA ? NSA : (n > MAX_NSA ? MAX_NSA : n);
}

int weight_stages(const TcLayer& L) {
  const size_t a = L.gather ? gather_stages(L) * gather_stage_bytes(L) + (L.wt ? kWtStage : 0)
                            : grid_a_stages(L) * a_stage_bytes(L);
  if (a + kSmemReserve >= kSmemLimit) return 0;
  size_t left = kSmemLimit - kSmemReserve - a;
  int n = (int)(left / ((size_t)L.nt * 128));
  return n < MAX_NSB ? n : MAX_NSB;
}

size_t smem_bytes(const TcLayer& L) {
  if (L.dxf && L.pair)
    return kDxfWBytes + (size_t)kD2NSA * 16 * 8 * pair_slab_rows(L) + kD2Xchg + kD2YStage + 256 + 128 +
           kSmemReserve;
  if (L.dxf) return kDxfWBytes + kDxfNSA * a_stage_bytes(L) + kDxfXchg + kDxfStage + 32 + kSmemReserve;
  if (L.gather)
    return gather_stages(L) * gather_stage_bytes(L) + (L.wt ? kWtStage : 0) + (size_t)weight_stages(L) * L.nt * 128 +
           kSmemReserve;
  return grid_a_stages(L) * a_stage_bytes(L) + (size_t)weight_stages(L) * L.nt * 128 + kSmemReserve;
}

int sm_count() { return device_sm_count(); }

template <int NT, int MSUB, bool FP8_IN, bool FP8_OUT>
tdm_status launch_t(const KParams& kp, size_t smem, cudaStream_t s) {
  auto kern = tc_conv_kernel<NT, MSUB, FP8_IN, FP8_OUT>;
  // Every tcgen05 CTA takes more than half an SM's shared memory, so two
  // TMEM-allocating CTAs never share an SM.
  size_t req = std::max<size_t>(smem, 120 * 1024);
  // The attribute is a per-device cap shared by every launch of this
  // instantiation: raise it to the full budget once per device.
  cudaError_t attr_err = raise_smem_cap(reinterpret_cast<const void*>(kern), (int)kSmemLimit);
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv_kernel)");
  int64_t grid = std::min<int64_t>(kp.total_tiles, sm_count());
  kern<<<(unsigned)std::max<int64_t>(grid, 1), kThreads, req, s>>>(kp);
  TDM_CHECK_LAUNCH("tc_conv_kernel");
  return TDM_OK;
}

template <int NT, int MSUB, bool FP8, bool XRUN, bool WT = false>
tdm_status launch_g(const KParams& kp, size_t smem, cudaStream_t s) {
  auto kern = tc_conv_gather_kernel<NT, MSUB, FP8, XRUN, WT>;
  size_t req = std::max<size_t>(smem, 120 * 1024);
  cudaError_t attr_err = raise_smem_cap(reinterpret_cast<const void*>(kern), (int)kSmemLimit);
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv_gather_kernel)");
  int64_t grid = std::min<int64_t>(kp.total_tiles, sm_count());
  kern<<<(unsigned)std::max<int64_t>(grid, 1), kGThreads, req, s>>>(kp);
  TDM_CHECK_LAUNCH("tc_conv_gather_kernel");
  return TDM_OK;
}

// Self-test of the bounded-wait path the tcgen05 kernels share.  One CTA of
// 64 threads allocates 32 TMEM columns the way the MMA warp does, lands one
// 64-byte bulk copy on barrier `full` (that wait completes), then waits on
// barrier `never`, on which nothing ever arrives.  That wait gives up after
// budget_ns and raises the device error word (DEV_TIMEOUT_MMA); the CTA then
// frees its TMEM and returns like a timed-out conv kernel.  out[0] = the copy
// landed, out[1] = the second wait ran out, out[2] = first copied word.
__device__ __align__(16) uint32_t g_selftest_src[16] = {0x5E1F7E57u, 1, 2, 3, 4, 5, 6, 7,
                                                        8, 9, 10, 11, 12, 13, 14, 15};

__global__ void __launch_bounds__(64, 1) wait_selftest_kernel(uint64_t budget_ns, int* err, int32_t* out) {
  __shared__ __align__(16) uint32_t buf[16];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5;
  const uint32_t full = ptx::smem_u32(&bars[0]), never = ptx::smem_u32(&bars[1]);
  if (threadIdx.x == 0) {
    ptx::mbar_init(full, 1);
    ptx::mbar_init(never, 1);
    ptx::fence_barrier_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(ptx::smem_u32(&tmem_slot), 32);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (threadIdx.x == 0) {
    ptx::mbar_arrive_expect_tx(full, sizeof(buf));
    ptx::bulk_g2s(ptx::smem_u32(buf), g_selftest_src, sizeof(buf), full);
    const bool copied = wait_or_flag(full, 0, err, DEV_TIMEOUT_PRODUCER, budget_ns);
    const bool timed_out = !wait_or_flag(never, 0, err, DEV_TIMEOUT_MMA, budget_ns);
    out[0] = copied ? 1 : 0;
    out[1] = timed_out ? 1 : 0;
    out[2] = copied ? (int32_t)buf[0] : 0;
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 32);
  }
}

// (N tile, M sub-tiles) shapes the gathered-row kernel is built for
bool gather_tile_built(int nt, int msub) {
  return (nt == 256 && (msub == 1 || msub == 2)) || (nt == 128 && msub == 2);
}

// CTA pairs of the pair form that can be resident at once on this device
// (clusters need both CTAs on one GPC; one CTA per SM), cached per device.
template <bool FP8_OUT, bool XPOOL, bool ZPOOL, bool YPOOL>
int dxf2_max_pairs(size_t smem) {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * (unsigned)(device_sm_count() / 2), 1, 1);
  cfg.blockDim = dim3(kD2Threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, tc_conv_dxf2_kernel<FP8_OUT, XPOOL, ZPOOL, YPOOL>, &cfg) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = device_sm_count() / 2;
  }
  cache[dev] = n;
  return n;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    cudaGetLastError();
  });
  return fn;
}

// The conv2 input as a 3-D byte tensor [8 chunks][plane rows / 2][32 B] (two
// 16-byte rows per line: every slab starts on an even row), read in boxes of
// one slab: [8][R / 2][32].  Lines past the plane are zero-filled.
tdm_status slab_tensor_map(const KParams& kp, CUtensorMap* map) {
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return fail(TDM_ERR_DEVICE, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[3] = {32, (cuuint64_t)(kp.act_cs / 32), 8};
  const cuuint64_t strides[2] = {32, (cuuint64_t)kp.act_cs};
  const cuuint32_t box[3] = {32, (cuuint32_t)kp.R / 2, 8};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<uint8_t*>(kp.act), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(TDM_ERR_DEVICE, "cuTensorMapEncodeTiled failed for the conv2 slab map");
  return TDM_OK;
}

template <bool FP8_OUT, bool XPOOL, bool ZPOOL, bool YPOOL>
tdm_status launch_dxf2(const KParams& kp, size_t smem, cudaStream_t s) {
  auto kern = tc_conv_dxf2_kernel<FP8_OUT, XPOOL, ZPOOL, YPOOL>;
  cudaError_t attr_err = raise_smem_cap(reinterpret_cast<const void*>(kern), (int)kSmemLimit);
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv_dxf2_kernel)");
  CUtensorMap map;
  tdm_status st = slab_tensor_map(kp, &map);
  if (st) return st;
  // persistent: no more pairs than fit at once, so every pair runs from the start
  const int max_pairs = dxf2_max_pairs<FP8_OUT, XPOOL, ZPOOL, YPOOL>(smem);
  const int64_t D3 = (int64_t)kp.D * kp.D * kp.D, B = kp.rows / D3;
  PairSched ps;
  ps.nyb = (kp.Do * kp.D + kD2Out - 1) / kD2Out;
  const int64_t cols = B * ps.nyb;
  // split the z walk only when the columns alone leave pairs idle
  const int64_t want = (4 * (int64_t)max_pairs + cols - 1) / cols;
  const int nseg0 = (int)std::max<int64_t>(1, std::min<int64_t>(kp.Do, want));
  ps.zs = (kp.Do + nseg0 - 1) / nseg0;
  if (ZPOOL) ps.zs += ps.zs & 1;  // whole z pairs per unit (Do is even)
  ps.nseg = (kp.Do + ps.zs - 1) / ps.zs;
  ps.nunits = (int)(cols * ps.nseg);
  const int64_t pairs = std::max<int64_t>(1, std::min<int64_t>(ps.nunits, max_pairs));
  kern<<<(unsigned)(2 * pairs), kD2Threads, smem, s>>>(kp, map, ps);
  TDM_CHECK_LAUNCH("tc_conv_dxf2_kernel");
  return TDM_OK;
}

// The pool's y-pair max at the pooled positions whose two rows the CTA-pair
// conv2 leaves in different CTA halves (a plane's rows are split into halves
// of 126 rows: pooled y = 4, where the 9-row blocks meet, and parts of the
// rows where a block's halves meet).  Both rows are in `in` x- and z-pooled,
// [b][z/2][y][x/2]; their max goes to the pooled output [b][z/2][y/2][x/2],
// whose other rows the pair kernel wrote.  E4M3 bytes of ReLU outputs order
// like the values, so a byte-wise max is the max-pool.
struct YCross {
  int n;            // crossing (y/2, x/2) positions of a pooled z plane
  uint16_t yx[64];  // y/2 << 8 | x/2
};

template <bool FP8>
__global__ __launch_bounds__(256) void pool_ycross_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out,
                                                          int64_t cs, int nchunks, int64_t planes, int Do,
                                                          const YCross c) {
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int64_t per = (int64_t)c.n * nchunks;
  if (i >= planes * per) return;
  const int64_t bz = i / per;  // b * Do/2 + z/2
  const int r = (int)(i - bz * per), j = r / c.n, e = r - j * c.n;
  const int yp = c.yx[e] >> 8, xp = c.yx[e] & 0xff, Dh = Do / 2;
  const uint8_t* src = in + (int64_t)j * cs;
  const uint4 a = __ldg(reinterpret_cast<const uint4*>(src + ((bz * Do + 2 * yp) * Dh + xp) * 16));
  const uint4 b = __ldg(reinterpret_cast<const uint4*>(src + ((bz * Do + 2 * yp + 1) * Dh + xp) * 16));
  uint4 o;
  if (FP8) {
    o.x = __vmaxu4(a.x, b.x);
    o.y = __vmaxu4(a.y, b.y);
    o.z = __vmaxu4(a.z, b.z);
    o.w = __vmaxu4(a.w, b.w);
  } else {
    const uint32_t* av = reinterpret_cast<const uint32_t*>(&a);
    const uint32_t* bv = reinterpret_cast<const uint32_t*>(&b);
    uint32_t* ov = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      __nv_bfloat162 m = __hmax2(*reinterpret_cast<const __nv_bfloat162*>(&av[k]),
                                 *reinterpret_cast<const __nv_bfloat162*>(&bv[k]));
      ov[k] = *reinterpret_cast<uint32_t*>(&m);
    }
  }
  *reinterpret_cast<uint4*>(out + (int64_t)j * cs + ((bz * Dh + yp) * Dh + xp) * 16) = o;
}

template <int MSUB, bool FP8_OUT, bool XPOOL>
tdm_status launch_dxf(const KParams& kp, size_t smem, cudaStream_t s) {
  auto kern = tc_conv_dxf_kernel<MSUB, FP8_OUT, XPOOL>;
  size_t req = std::max<size_t>(smem, 120 * 1024);
  cudaError_t attr_err = raise_smem_cap(reinterpret_cast<const void*>(kern), (int)kSmemLimit);
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv_dxf_kernel)");
  // an even grid keeps every CTA on one half of the output channels
  int64_t grid = std::min<int64_t>(kp.total_tiles, sm_count() & ~1);
  kern<<<(unsigned)std::max<int64_t>(grid, 2), kThreads, req, s>>>(kp);
  TDM_CHECK_LAUNCH("tc_conv_dxf_kernel");
  return TDM_OK;
}

}  // namespace

tdm_status launch_pool_ycross(const TcLayer& L, const uint8_t* in, int64_t cs, int B, uint8_t* out, cudaStream_t s) {
  TDM_REQUIRE(L.dxf && L.pair && L.Do % 2 == 0 && L.Do / 2 < 256, "pool: the y-pair finish follows the CTA-pair conv2");
  TDM_REQUIRE(in && out && (cs & 15) == 0 && B >= 0, "pool: bad arguments");
  YCross c{};
  const int Dh = L.Do / 2;
  for (int yp = 0; yp < Dh; ++yp)
    for (int xp = 0; xp < Dh; ++xp) {
      const int pp = 2 * yp * L.D + 2 * xp;  // the even row's index in its z plane; its partner is pp + D
      if (pp / kDxfSub != (pp + L.D) / kDxfSub) {
        TDM_REQUIRE(c.n < 64, "pool: too many crossing y pairs");
        c.yx[c.n++] = (uint16_t)(yp << 8 | xp);
      }
    }
  if (B == 0 || c.n == 0) return TDM_OK;
  const int nchunks = L.fp8_out ? 4 : 8;
  const int64_t planes = (int64_t)B * Dh, n = planes * c.n * nchunks;
  if (L.fp8_out)
    pool_ycross_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, cs, nchunks, planes, L.Do, c);
  else
    pool_ycross_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, cs, nchunks, planes, L.Do, c);
  TDM_CHECK_LAUNCH("pool_ycross_kernel");
  return TDM_OK;
}

// conv1 of B patches into conv2's chunk-planar BF16 input (out_cs bytes
// between its 8 chunks); weights packed as the conv1 GEMM layer's.
tdm_status launch_conv1_tc(const float* patches, int B, const TcLayer& L, uint8_t* out, int64_t out_cs,
                           cudaStream_t s) {
  TDM_REQUIRE(L.wpk && L.bias && L.nt == 64 && L.cin == 32, "conv1: weights not packed for the tensor-core form");
  TDM_REQUIRE((reinterpret_cast<uintptr_t>(out) & 15) == 0 && (out_cs & 15) == 0, "conv1: output must be 16-byte aligned");
  C1Params p;
  p.patches = patches;
  p.rows = (int64_t)B * 21952;
  p.wpk = L.wpk;
  p.bias = L.bias;
  p.out = out;
  p.out_cs = out_cs;
  p.tiles = (int64_t)B * kC1TilesPerPatch;
  p.err = device_error_word();
  if (!p.err) return fail(TDM_ERR_DEVICE, "device error word unavailable");
  if (p.rows == 0) return TDM_OK;
  TDM_REQUIRE((reinterpret_cast<uintptr_t>(patches) & 15) == 0, "conv1: patches must be 16-byte aligned");
  const size_t smem = kC1W + kC1NSA * kC1Stage + 2 * kC1PlaneSpan * 4 + 256;
  cudaError_t attr_err = raise_smem_cap(reinterpret_cast<const void*>(tc_conv1_kernel), (int)kSmemLimit);
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv1_kernel)");
  const int64_t grid = std::min<int64_t>(p.tiles, sm_count());
  tc_conv1_kernel<<<(unsigned)grid, kC1Threads, std::max<size_t>(smem, 120 * 1024), s>>>(p);
  TDM_CHECK_LAUNCH("tc_conv1_kernel");
  return TDM_OK;
}

tdm_status launch_wait_selftest(uint64_t budget_ns, int32_t* out, cudaStream_t s) {
  int* err = device_error_word();
  if (!err) return fail(TDM_ERR_DEVICE, "device error word unavailable");
  wait_selftest_kernel<<<1, 64, 0, s>>>(budget_ns, err, out);
  TDM_CHECK_LAUNCH("wait_selftest_kernel");
  return TDM_OK;
}

#ifdef TDM_WAIT_STATS
}  // namespace tdm
extern "C" int tdm_debug_wait_stats(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, tdm::g_wait_stats, sizeof(unsigned long long) * 16) != cudaSuccess) return 1;
  if (reset) {
    unsigned long long z[16] = {};
    if (cudaMemcpyToSymbol(tdm::g_wait_stats, z, sizeof(z)) != cudaSuccess) return 1;
  }
  return 0;
}
namespace tdm {
#endif

int64_t tc_tail_rows(const TcLayer& L) {
  return (int64_t)(L.nz > 1 ? 2 * L.D * L.D : 0) + slab_rows(L) + 8;
}

bool tc_layer_fits(const TcLayer& L) {
  if (L.dxf && L.pair)  // the pair covers both channel halves and 2 x 126 rows: tile (32, 2) only
    return L.nt == kDxfNt && L.msub == 2 && L.cin == 64 && L.cout == 2 * kDxfNt && L.nz == 3 && L.nyx == 9 &&
           !L.fp8_in && smem_bytes(L) <= kSmemLimit;
  if (L.dxf)
    return L.nt == kDxfNt && (L.msub == 1 || L.msub == 2) && L.cin == 64 && L.cout == 2 * kDxfNt && L.nz == 3 &&
           L.nyx == 9 && !L.fp8_in && smem_bytes(L) <= kSmemLimit;
  if (L.gather)
    return L.nz == 3 && L.nyx == 9 && L.fp8_in == L.fp8_out && gather_tile_built(L.nt, L.msub) &&
           L.cout % L.nt == 0 && weight_stages(L) >= 2 && smem_bytes(L) <= kSmemLimit &&
           (!L.wt || (L.nt == 128 && L.msub == 2 && L.cout == 128 && L.out_mode == TC_OUT_C8_CONV));
  return L.nt > 0 && L.msub > 0 && L.cout % L.nt == 0 && 2 * L.msub * L.nt <= 512 && weight_stages(L) >= 2 &&
         smem_bytes(L) <= kSmemLimit;
}

bool tc_pair_form_applies(const TcLayer& L, int64_t rows) {
  return L.dxf && L.pair && rows <= kPairMaxRows && rows % ((int64_t)L.D * L.D * L.D) == 0;
}

tdm_status launch_tc_layer(const TcLayer& L, const TcArgs& a, cudaStream_t s) {
  KParams kp;
  kp.act = a.act;
  kp.act_cs = a.act_cs;
  kp.rows = a.rows;
  kp.wpk = L.wpk;
  kp.bias = L.bias;
  kp.wscale = L.wscale;
  kp.in_scale = a.in_scale;
  kp.out_qinv = a.out_qinv;
  kp.out = a.out;
  kp.out_cs = a.out_cs;
  kp.out2 = a.out2;
  kp.D = L.D;
  kp.Do = L.Do;
  kp.nz = L.nz;
  kp.nyx = L.nyx;
  kp.kgroups = L.kgroups;
  kp.cpg = chunks_per_group(L);
  kp.cout = L.cout;
  kp.out_mode = L.out_mode;
  kp.relu = L.relu;
  kp.R = slab_rows(L);
  kp.err = device_error_word();
  if (!kp.err) return fail(TDM_ERR_DEVICE, "device error word unavailable");
  if (L.dxf && L.pair && !tc_pair_form_applies(L, a.rows)) {
    // slab rows are 32-bit tensor coordinates and units are whole patches:
    // other inputs take the single-CTA form (same bits)
    TDM_REQUIRE(!a.zpool && !a.out2, "tc layer: the z- and y-pair max need the CTA-pair form");
    TcLayer L1 = L;
    L1.pair = false;
    return launch_tc_layer(L1, a, s);
  }
  if (L.dxf && L.pair) {
    TDM_REQUIRE(tc_layer_fits(L), "tc layer: unsupported dx-fused pair tile");
    TDM_REQUIRE((reinterpret_cast<uintptr_t>(a.act) & 15) == 0 && (a.act_cs & 15) == 0 &&
                    (reinterpret_cast<uintptr_t>(L.wpk) & 15) == 0 && (reinterpret_cast<uintptr_t>(a.out) & 15) == 0 &&
                    (a.out_cs & 15) == 0,
                "tc layer: operands must be 16-byte aligned");
    if (a.rows == 0) return TDM_OK;
    TDM_REQUIRE(!a.xpool || (L.D % 2 == 0 && L.Do % 2 == 0), "tc layer: x-pooled output needs even extents");
    kp.R = pair_slab_rows(L);
    kp.ntiles = 1;
    kp.nsb = 0;
    kp.total_tiles = (a.rows + kD2Out - 1) / kD2Out;
    const size_t smem = smem_bytes(L);
    TDM_REQUIRE(!a.zpool || (a.xpool && L.Do % 2 == 0), "tc layer: a z-pooled output needs the x-pooled form, even Do");
    TDM_REQUIRE(!a.out2 || (a.zpool && (reinterpret_cast<uintptr_t>(a.out2) & 15) == 0),
                "tc layer: the y-pooled output needs the z-pooled form and 16-byte alignment");
    if (L.fp8_out) {
      if (a.zpool)
        return a.out2 ? launch_dxf2<true, true, true, true>(kp, smem, s) : launch_dxf2<true, true, true, false>(kp, smem, s);
      return a.xpool ? launch_dxf2<true, true, false, false>(kp, smem, s)
                     : launch_dxf2<true, false, false, false>(kp, smem, s);
    }
    if (a.zpool)
      return a.out2 ? launch_dxf2<false, true, true, true>(kp, smem, s) : launch_dxf2<false, true, true, false>(kp, smem, s);
    return a.xpool ? launch_dxf2<false, true, false, false>(kp, smem, s)
                   : launch_dxf2<false, false, false, false>(kp, smem, s);
  }
  if (L.dxf) {
    TDM_REQUIRE(tc_layer_fits(L), "tc layer: unsupported dx-fused tile");
    TDM_REQUIRE((reinterpret_cast<uintptr_t>(a.act) & 15) == 0 && (a.act_cs & 15) == 0 &&
                    (reinterpret_cast<uintptr_t>(L.wpk) & 15) == 0,
                "tc layer: operands must be 16-byte aligned");
    if (a.rows == 0) return TDM_OK;
    const int64_t mout = (int64_t)L.msub * kDxfSub;
    kp.ntiles = 2;
    kp.nsb = 0;
    kp.total_tiles = ((a.rows + mout - 1) / mout) * 2;
    const size_t smem = smem_bytes(L);
    TDM_REQUIRE(!a.xpool || (L.D % 2 == 0 && L.Do % 2 == 0), "tc layer: x-pooled output needs even extents");
#define TDM_DXF(MS_, F8_)                                                                       \
    return a.xpool ? launch_dxf<MS_, F8_, true>(kp, smem, s) : launch_dxf<MS_, F8_, false>(kp, smem, s)
    if (L.msub == 2) {
      if (L.fp8_out) TDM_DXF(2, true);
      TDM_DXF(2, false);
    }
    if (L.fp8_out) TDM_DXF(1, true);
    TDM_DXF(1, false);
#undef TDM_DXF
  }
  if (L.gather) {
    TDM_REQUIRE(tc_layer_fits(L), "tc layer: unsupported gathered-row tile");
    TDM_REQUIRE((reinterpret_cast<uintptr_t>(a.act) & 15) == 0 && (a.act_cs & 15) == 0 &&
                    (reinterpret_cast<uintptr_t>(L.wpk) & 15) == 0,
                "tc layer: operands must be 16-byte aligned");
    const int64_t D3 = (int64_t)L.D * L.D * L.D;
    TDM_REQUIRE(a.rows % D3 == 0, "tc layer: input rows must be whole patches");
    // M = valid output positions, or in the x-run form whole x runs of them
    kp.rows = a.rows / D3 * L.Do * L.Do * (L.xrun ? L.D : L.Do);
    if (kp.rows == 0) return TDM_OK;
    kp.nsb = weight_stages(L);
    const int64_t mcta = (int64_t)L.msub * 128;
    kp.ntiles = L.cout / L.nt;
    kp.total_tiles = ((kp.rows + mcta - 1) / mcta) * kp.ntiles;
    const size_t smem = smem_bytes(L);
    const bool f8 = L.fp8_in;
#define TDM_G_CASE(NT_, MS_)                                                              \
  if (L.nt == NT_ && L.msub == MS_) {                                                     \
    if (L.xrun) return f8 ? launch_g<NT_, MS_, true, true>(kp, smem, s) : launch_g<NT_, MS_, false, true>(kp, smem, s); \
    return f8 ? launch_g<NT_, MS_, true, false>(kp, smem, s) : launch_g<NT_, MS_, false, false>(kp, smem, s);           \
  }
    if (L.wt) {
      if (f8) return L.xrun ? launch_g<128, 2, true, true, true>(kp, smem, s) : launch_g<128, 2, true, false, true>(kp, smem, s);
      return L.xrun ? launch_g<128, 2, false, true, true>(kp, smem, s) : launch_g<128, 2, false, false, true>(kp, smem, s);
    }
    TDM_G_CASE(256, 2)
    TDM_G_CASE(256, 1)
    TDM_G_CASE(128, 2)
#undef TDM_G_CASE
    return fail(TDM_ERR_UNSUPPORTED, "tc layer: unsupported gathered-row tile");
  }
  kp.nsb = weight_stages(L);
  kp.nsa = grid_a_stages(L);
  kp.ksplit = L.ksplit > 1 ? L.ksplit : 1;
  kp.part = a.part;
  TDM_REQUIRE(kp.ksplit == 1 || (L.nz == 1 && L.nyx == 1 && L.kgroups % kp.ksplit == 0 && a.part &&
                                 (L.out_mode == TC_OUT_F32_ROWS || (L.out_mode == TC_OUT_C8_ROWS && !L.fp8_out))),
              "tc layer: split-K needs a plain GEMM, K groups divisible by the splits, a partial buffer, F32 or BF16 rows");
  TDM_REQUIRE(kp.nsb >= 2, "tc layer: shared-memory plan leaves fewer than 2 weight stages");
  TDM_REQUIRE(smem_bytes(L) <= kSmemLimit, "tc layer: shared-memory plan exceeds 227 KB");
  TDM_REQUIRE(L.cout % L.nt == 0, "tc layer: cout must be a multiple of the N tile");
  TDM_REQUIRE((reinterpret_cast<uintptr_t>(a.act) & 15) == 0 && (a.act_cs & 15) == 0 &&
                  (reinterpret_cast<uintptr_t>(L.wpk) & 15) == 0,
              "tc layer: operands must be 16-byte aligned");
  if (a.rows == 0) return TDM_OK;
  const int64_t mcta = (int64_t)L.msub * 128;
  const int64_t mtiles = (a.rows + mcta - 1) / mcta;
  kp.ntiles = L.cout / L.nt;
  kp.total_tiles = mtiles * kp.ntiles * kp.ksplit;
  const size_t smem = smem_bytes(L);
  const bool f8i = L.fp8_in, f8o = L.fp8_out;
  if (kp.ksplit > 1) {
    tdm_status st = TDM_OK;
#define TDM_TC_SPLIT(NT_, MS_)                                                                         \
    if (L.nt == NT_ && L.msub == MS_) st = f8i ? launch_t<NT_, MS_, true, false>(kp, smem, s)          \
                                               : launch_t<NT_, MS_, false, false>(kp, smem, s);       \
    else
    TDM_TC_SPLIT(64, 4) TDM_TC_SPLIT(64, 2) TDM_TC_SPLIT(128, 2) TDM_TC_SPLIT(128, 1) TDM_TC_SPLIT(256, 1)
    return fail(TDM_ERR_UNSUPPORTED, "tc layer: unsupported (nt, msub) tile");
#undef TDM_TC_SPLIT
    if (st) return st;
    const int64_t n = a.rows * (L.cout / 8);
    if (f8i)
      splitk_reduce_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
          a.part, kp.ksplit, a.rows, L.cout, L.bias, L.wscale, a.in_scale, L.relu, L.out_mode, a.out, a.out_cs);
    else
      splitk_reduce_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
          a.part, kp.ksplit, a.rows, L.cout, L.bias, L.wscale, a.in_scale, L.relu, L.out_mode, a.out, a.out_cs);
    TDM_CHECK_LAUNCH("splitk_reduce_kernel");
    return TDM_OK;
  }
#define TDM_TC_CASE(NT_, MS_)                                                                  \
  if (L.nt == NT_ && L.msub == MS_) {                                                          \
    if (f8i && f8o) return launch_t<NT_, MS_, true, true>(kp, smem, s);                        \
    if (f8i) return launch_t<NT_, MS_, true, false>(kp, smem, s);                              \
    if (f8o) return launch_t<NT_, MS_, false, true>(kp, smem, s);                              \
    return launch_t<NT_, MS_, false, false>(kp, smem, s);                                      \
  }
  TDM_TC_CASE(64, 4)
  TDM_TC_CASE(64, 2)
  TDM_TC_CASE(128, 2)
  TDM_TC_CASE(128, 1)
  TDM_TC_CASE(256, 1)
#undef TDM_TC_CASE
  return fail(TDM_ERR_UNSUPPORTED, "tc layer: unsupported (nt, msub) tile");
}

void pack_dxf_weights(const TcLayer& L, const float* w, std::vector<uint8_t>* out) {
  out->assign((size_t)2 * kDxfWBytes, 0);
  for (int h = 0; h < 2; ++h)
    for (int b = 0; b < 9; ++b)  // b = dz * 3 + dy
      for (int j = 0; j < 8; ++j)
        for (int n = 0; n < kDxfN; ++n) {
          const int dx = n / kDxfNt, co = h * kDxfNt + n % kDxfNt;
          for (int e = 0; e < 8; ++e) {
            const int ci = j * 8 + e;
            const __nv_bfloat16 v = __float2bfloat16_rn(w[((size_t)co * L.cin + ci) * 27 + b * 3 + dx]);
            std::memcpy(out->data() + (size_t)h * kDxfWBytes + (size_t)b * kDxfBlock + ((size_t)j * kDxfN + n) * 16 +
                            2 * e,
                        &v, 2);
          }
        }
}

// Weight blocks: for ntile, zt, cg, yx -> [chunk j][n in nt][16 bytes], where
// chunk j of group cg holds K elements [cg*kg + j*e, +e) of that tap (e = 8
// BF16 or 16 E4M3 per chunk, kg = e * chunks per group).  `w` is Marvin's
// [cout][cin][taps] float; for a GEMM (nz = nyx = 1) with gemm_taps > 1 the K
// index is tap*cin + c (conv8 on the flattened 3^3 x 512 input).
void pack_tc_weights(const TcLayer& L, const float* w, int gemm_taps, std::vector<uint8_t>* out,
                     std::vector<float>* scales) {
  const int taps = L.nz * L.nyx;
  const int e = L.fp8_in ? 16 : 8;
  const int cpg = chunks_per_group(L);
  const int kg = e * cpg;
  const int ntiles = L.cout / L.nt;
  const size_t blk = (size_t)L.nt * 128;
  const int tapsK = taps > 1 ? taps : gemm_taps;  // taps in Marvin's weight layout
  out->assign((size_t)ntiles * taps * L.kgroups * blk, 0);
  scales->assign(L.cout, 1.0f);
  if (L.fp8_in) {
    for (int n = 0; n < L.cout; ++n) {
      float mx = 0.0f;
      for (size_t i = 0; i < (size_t)L.cin * tapsK; ++i) mx = std::max(mx, std::fabs(w[(size_t)n * L.cin * tapsK + i]));
      (*scales)[n] = mx > 0.0f ? mx / 448.0f : 1.0f;
    }
  }
  for (int nt = 0; nt < ntiles; ++nt)
    for (int zt = 0; zt < L.nz; ++zt)
      for (int cg = 0; cg < L.kgroups; ++cg)
        for (int yx = 0; yx < L.nyx; ++yx) {
          uint8_t* b = out->data() + ((((size_t)nt * L.nz + zt) * L.kgroups + cg) * L.nyx + yx) * blk;
          for (int j = 0; j < cpg; ++j)
            for (int n = 0; n < L.nt; ++n)
              for (int q = 0; q < e; ++q) {
                int kidx = cg * kg + j * e + q;  // K index within this tap (conv) or overall (GEMM)
                int co = nt * L.nt + n;
                float v;
                if (taps > 1) {
                  v = w[((size_t)co * L.cin + kidx) * taps + (zt * L.nyx + yx)];
                } else {
                  int tap = kidx / L.cin, c = kidx % L.cin;
                  v = w[((size_t)co * L.cin + c) * tapsK + tap];
                }
                uint8_t* dst = b + (size_t)j * L.nt * 16 + (size_t)n * 16;
                if (L.fp8_in) {
                  __nv_fp8_e4m3 f(v / (*scales)[co]);
                  std::memcpy(dst + q, &f, 1);
                } else {
                  __nv_bfloat16 h = __float2bfloat16_rn(v);
                  std::memcpy(dst + 2 * q, &h, 2);
                }
              }
        }
}

}  // namespace tdm

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
#include <cuda_fp8.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace tdm {
namespace {

constexpr int NSA = 2;      // A slab stages
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
  int D, Do, nz, nyx, kgroups, cpg, cout, out_mode, relu, R, nsb, ntiles;
  int64_t total_tiles;
  int* err;
};

__host__ __device__ constexpr uint32_t tmem_cols_for(int c) {
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

__device__ __forceinline__ bool aborted(const int* err) { return *reinterpret_cast<const volatile int*>(err) != 0; }

__device__ __forceinline__ bool wait_or_flag(uint32_t bar, uint32_t parity, int* err, int code) {
  if (ptx::mbar_try_wait(bar, parity)) return true;
  uint64_t t0 = ptx::globaltimer_ns();
  uint32_t spins = 0;
  while (true) {
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if ((++spins & 255u) == 0) {
      if (aborted(err)) return false;
      if (ptx::globaltimer_ns() - t0 > kWaitBudgetNs) {
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
__device__ unsigned long long g_wait_stats[8];
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
  const int64_t r0 = m0 % D3;
  return !(r0 >= (int64_t)p.Do * D2 && r0 + mcta <= D3);
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
  uint8_t* sB = smem + NSA * a_stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + (size_t)nsb * b_stage);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * NSA + 2 * MAX_NSB + 5);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (!__syncthreads_and(aborted(p.err) ? 0 : 1)) return;  // another CTA already failed

  const uint32_t fullA = ptx::smem_u32(bars), emptyA = fullA + 8 * NSA;
  const uint32_t fullB = emptyA + 8 * NSA, emptyB = fullB + 8 * MAX_NSB;
  const uint32_t accFull = emptyB + 8 * MAX_NSB, accEmpty = accFull + 16, done = accEmpty + 16;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NSA; ++i) { ptx::mbar_init(fullA + 8 * i, 1); ptx::mbar_init(emptyA + 8 * i, 1); }
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
      int armedA[NSA], armedB[MAX_NSB];  // parity of each stage's last arming, -1 = never
      for (int i = 0; i < NSA; ++i) armedA[i] = -1;
      for (int i = 0; i < MAX_NSB; ++i) armedB[i] = -1;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t / p.ntiles) * MCTA;
        const int nt = (int)(t % p.ntiles);
        if (!tile_has_work(p, m0, MCTA)) continue;
        for (int zt = 0; zt < p.nz && ok; ++zt) {
          for (int cg = 0; cg < p.kgroups && ok; ++cg) {
            if (!TDM_TIMED_WAIT(3, wait_or_flag(emptyA + 8 * sa, pha ^ 1, p.err, DEV_TIMEOUT_PRODUCER))) { ok = false; break; }
            ptx::mbar_arrive_expect_tx(fullA + 8 * sa, a_stage);
            armedA[sa] = (int)pha;
            const uint8_t* src = p.act + (int64_t)cg * p.cpg * p.act_cs + (m0 + zt * plane) * 16;
            for (int j = 0; j < p.cpg; ++j)
              ptx::bulk_g2s(sA_u + sa * a_stage + j * R * 16, src + j * p.act_cs, R * 16, fullA + 8 * sa);
            if (++sa == NSA) { sa = 0; pha ^= 1; }
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
      for (int i = 0; i < NSA; ++i)
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
      uint32_t j = 0;  // tiles done by this CTA
      for (int64_t t = blockIdx.x; t < p.total_tiles && ok; t += gridDim.x) {
        const int64_t m0 = (t / p.ntiles) * MCTA;
        if (!tile_has_work(p, m0, MCTA)) continue;
        const uint32_t buf = j & 1u, use = j >> 1;
        if (!TDM_TIMED_WAIT(0, wait_or_flag(accEmpty + 8 * buf, (use & 1u) ^ 1u, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
        ptx::tc_fence_after();
        const uint32_t dbase = tmem + buf * ACC_COLS;
        uint32_t accumulate = 0;
        for (int zt = 0; zt < p.nz && ok; ++zt) {
          for (int cg = 0; cg < p.kgroups && ok; ++cg) {
            if (!TDM_TIMED_WAIT(1, wait_or_flag(fullA + 8 * sa, pha, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
            ptx::tc_fence_after();
            const uint32_t aBase = sA_u + sa * a_stage;
            for (int yx = 0; yx < p.nyx; ++yx) {
              if (!TDM_TIMED_WAIT(2, wait_or_flag(fullB + 8 * sb, phb, p.err, DEV_TIMEOUT_MMA))) { ok = false; break; }
              ptx::tc_fence_after();
              const uint32_t bBase = sB_u + sb * b_stage;
              const int off = (p.nyx > 1) ? (yx / 3) * p.D + (yx % 3) : 0;
              for (int kk = 0; kk < p.cpg / 2; ++kk) {
                const uint64_t bdesc = ptx::smem_desc(bBase + (2 * kk) * NT * 16, NT * 16, 128);
#pragma unroll
                for (int i = 0; i < MSUB; ++i) {
                  const uint64_t adesc =
                      ptx::smem_desc(aBase + (2 * kk) * lboA + (uint32_t)(i * 128 + off) * 16u, lboA, 128);
                  if (FP8_IN) ptx::mma_f8(dbase + i * NT, adesc, bdesc, idesc, accumulate);
                  else ptx::mma_f16(dbase + i * NT, adesc, bdesc, idesc, accumulate);
                }
                accumulate = 1;
              }
              ptx::mma_commit(emptyB + 8 * sb);
              if (++sb == nsb) { sb = 0; phb ^= 1; }
            }
            ptx::mma_commit(emptyA + 8 * sa);
            if (++sa == NSA) { sa = 0; pha ^= 1; }
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
      const int64_t m0 = (t / p.ntiles) * MCTA;
      const int n0 = (int)(t % p.ntiles) * NT;
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
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            float a = v[e];
            if (FP8_IN) a = a * (p.in_scale * __ldg(p.wscale + n + e));
            a += __ldg(p.bias + n + e);
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

int slab_rows(const TcLayer& L) {
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

int weight_stages(const TcLayer& L) {
  size_t left = kSmemLimit - kSmemReserve - NSA * a_stage_bytes(L);
  int n = (int)(left / ((size_t)L.nt * 128));
  return n < MAX_NSB ? n : MAX_NSB;
}

size_t smem_bytes(const TcLayer& L) {
  return NSA * a_stage_bytes(L) + (size_t)weight_stages(L) * L.nt * 128 + kSmemReserve;
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
  }
  return n;
}

template <int NT, int MSUB, bool FP8_IN, bool FP8_OUT>
tdm_status launch_t(const KParams& kp, size_t smem, cudaStream_t s) {
  auto kern = tc_conv_kernel<NT, MSUB, FP8_IN, FP8_OUT>;
  // Every tcgen05 CTA takes more than half an SM's shared memory, so two
  // TMEM-allocating CTAs never share an SM.
  size_t req = std::max<size_t>(smem, 120 * 1024);
  // The attribute is a cap shared by every launch of this instantiation (from
  // any host thread): raise it once to the full budget.
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [&] {
    attr_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
  });
  if (attr_err != cudaSuccess) return cuda_status(attr_err, "cudaFuncSetAttribute(tc_conv_kernel)");
  int64_t grid = std::min<int64_t>(kp.total_tiles, sm_count());
  kern<<<(unsigned)std::max<int64_t>(grid, 1), kThreads, req, s>>>(kp);
  TDM_CHECK_LAUNCH("tc_conv_kernel");
  return TDM_OK;
}

}  // namespace

#ifdef TDM_WAIT_STATS
}  // namespace tdm
extern "C" int tdm_debug_wait_stats(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, tdm::g_wait_stats, sizeof(unsigned long long) * 8) != cudaSuccess) return 1;
  if (reset) {
    unsigned long long z[8] = {};
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
  return L.nt > 0 && L.msub > 0 && L.cout % L.nt == 0 && 2 * L.msub * L.nt <= 512 && weight_stages(L) >= 2 &&
         smem_bytes(L) <= kSmemLimit;
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
  kp.nsb = weight_stages(L);
  kp.err = device_error_word();
  if (!kp.err) return fail(TDM_ERR_DEVICE, "device error word unavailable");
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
  kp.total_tiles = mtiles * kp.ntiles;
  const size_t smem = smem_bytes(L);
  const bool f8i = L.fp8_in, f8o = L.fp8_out;
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

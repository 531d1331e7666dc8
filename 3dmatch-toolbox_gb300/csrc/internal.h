// Launchers shared between translation units of libtdm (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "tdm.h"

namespace tdm {

// ---- conv_simt.cu ----
tdm_status launch_conv1(const float* patches, int B, const float* w, const float* bias, bool bf16_out, void* out,
                        int64_t out_cs, cudaStream_t s);
// BF16 tensor-core form of conv1: 27 taps (padded to 32) per output position.
tdm_status launch_conv_f32(const float* in, int B, int D, int C, int ks, const float* w, const float* bias, int K,
                           bool relu, float* out, cudaStream_t s);
tdm_status launch_pool_f32(const float* in, int B, int D, int C, float* out, cudaStream_t s);
// x_pooled: the input's x extent is already D/2 (max of x pairs, from conv2's epilogue);
// z_pooled (with x_pooled): so is its z extent (max of z pairs)
tdm_status launch_pool_c16_u8(const uint8_t* in, int64_t in_cs, int B, int D, int nchunks, uint8_t* out,
                              int64_t out_cs, cudaStream_t s, bool x_pooled = false, bool z_pooled = false);
tdm_status launch_pool_c8(const uint8_t* in, int64_t in_cs, int B, int D, int nchunks, uint8_t* out, int64_t out_cs,
                          cudaStream_t s, bool x_pooled = false, bool z_pooled = false);

// ---- conv_tc.cu: tcgen05 implicit-GEMM convolution / GEMM ----
// Output layouts of the tensor-core epilogue.
enum TcOutMode : int {
  TC_OUT_C8_CONV = 0,   // chunk-planar, re-linearised from the D^3 input grid to the Do^3 output grid
  TC_OUT_C8_TAPS = 1,   // chunk-planar GEMM operand: K index = tap*Cout + c, row = patch (conv7 -> conv8)
  TC_OUT_C8_ROWS = 2,   // chunk-planar, row = input row (GEMM outputs)
  TC_OUT_F32_ROWS = 3,  // float [rows][Cout]
};

struct TcLayer {
  // geometry
  int cin, cout;
  int D, Do;      // input / output spatial extent (conv); D = 1 for a GEMM
  int nz, nyx;    // tap structure: (3, 9) for 3x3x3 conv, (1, 1) for a GEMM
  int kgroups;    // 128-byte K groups per tap (cin*elem/128)
  int nt, msub;   // N tile and number of 128-row M sub-tiles per CTA
  int out_mode;
  int relu;
  bool fp8_in;    // operands are E4M3 (kind::f8f6f4)
  bool fp8_out;   // epilogue writes E4M3 (chunk of 16 channels per 16 bytes)
  // dx-fused form (a 3x3x3 conv with 64 BF16 inputs and 64 outputs, i.e.
  // conv2): the three dx taps of one (dz, dy) form a single N = 3 * nt MMA
  // and the epilogue adds the dx = 1, 2 partial sums from the next one and
  // two rows; nt = 32 output channels per CTA (two halves), weights resident
  // in shared memory, msub sub-tiles of 128 rows giving 126 outputs each.
  bool dxf = false;
  // dx-fused on a CTA pair (cta_group::2): one M = 256, N = 192 MMA per K step
  // covers 256 rows and all 64 output channels (each CTA holds one weight half)
  bool pair = false;
  // gathered-row form (3x3x3 convs): M runs over the valid output positions
  // only and gather warps copy each tap's A rows into shared memory, instead
  // of the grid form's rows for every input position.
  bool gather = false;
  // x-run variant of the gathered form: M rows keep whole input x runs (D per
  // (b, z, y)), so one staged A operand serves the three dx taps by a row
  // shift; D/Do of the rows are computed for Do outputs.
  bool xrun = false;
  // weights as the A operand (128 BF16 output channels, gathered forms): one
  // 128 x 256 x 16 MMA per K step over both row sub-tiles
  bool wt = false;
  // K splits of a plain GEMM (conv8): each tile accumulates one K range into
  // FP32 partials and a reduce pass adds them in order (more CTAs for a
  // 2,048-row GEMM with K = 13,824)
  int ksplit = 1;
  // device data
  uint8_t* wpk;   // packed weights, blocks [ntile][zt][cg][yx] of nt*128 bytes
  float* bias;    // [cout]
  float* wscale;  // per-output-channel dequantisation scale (FP8) or null
};

struct TcArgs {
  const uint8_t* act;
  int64_t act_cs;  // bytes between input chunks
  int64_t rows;    // input rows (B*D^3 conv; B GEMM)
  uint8_t* out;
  int64_t out_cs;  // bytes between output chunks
  float in_scale;  // FP8: activation dequantisation scale of the input
  float out_qinv;  // FP8 output: 1/scale used to quantise
  bool xpool = false;  // dx-fused conv2: write the max of each x pair (x extent Do/2)
  bool zpool = false;  // with xpool, CTA-pair form only: also the max of each z pair (z extent Do/2)
  // with zpool: the pooled rows ([b][z/2][y/2][x/2], out_cs between chunks) of
  // the y pairs whose rows share a CTA half go here; `out` keeps the x- and
  // z-pooled rows of the others, which launch_pool_ycross finishes
  uint8_t* out2 = nullptr;
  float* part = nullptr;  // split-K partial sums, [ksplit][rows][cout] FP32
};

// Rows of slack a chunk-planar input needs after its last row for layer L.
int64_t tc_tail_rows(const TcLayer& L);
tdm_status launch_tc_layer(const TcLayer& L, const TcArgs& a, cudaStream_t s);
// Whether launch_tc_layer runs layer L over `rows` input rows in the CTA-pair
// form (which alone can take the z-pair max, TcArgs::zpool).
bool tc_pair_form_applies(const TcLayer& L, int64_t rows);
// The y-pair max of the pooled positions the CTA-pair conv2 (layer L, y-pooled
// into `out`) left to a pool pass: reads its x- and z-pooled rows in `in`.
tdm_status launch_pool_ycross(const TcLayer& L, const uint8_t* in, int64_t cs, int B, uint8_t* out, cudaStream_t s);
// conv1 with its im2col operand built in shared memory (L = the conv1 GEMM
// layer's packed weights and bias); writes conv2's chunk-planar BF16 input.
tdm_status launch_conv1_tc(const float* patches, int B, const TcLayer& L, uint8_t* out, int64_t out_cs,
                           cudaStream_t s);
// One-CTA kernel that runs the tcgen05 kernels' bounded wait into its time
// limit on purpose (out: 3 int32 on the device); raises the error word.
tdm_status launch_wait_selftest(uint64_t budget_ns, int32_t* out, cudaStream_t s);
// Whether layer L's (nt, msub) tile fits the shared-memory plan and TMEM.
bool tc_layer_fits(const TcLayer& L);
// Packs Marvin-layout weights [cout][cin][taps] (taps = nz*nyx, or the GEMM
// K flattening for conv8) into the tcgen05 block layout; returns host bytes.
void pack_tc_weights(const TcLayer& L, const float* w, int gemm_taps, std::vector<uint8_t>* out,
                     std::vector<float>* scales);
// Weights of a dx-fused layer: [half][dz*3+dy][chunk][dx*nt + c][16 bytes].
void pack_dxf_weights(const TcLayer& L, const float* w, std::vector<uint8_t>* out);

// TDF workspace bytes enough for any grid of at most V voxels: the x rows of
// the two byte arrays are padded to 4 and a grid is at least 31 voxels wide.
inline size_t tdf_workspace_cap(int64_t V) { return 2 * ((size_t)V * 34 / 31 + 1024); }

// Net properties the batched form needs (net.cu).
int net_max_batch(const tdm_net* net);
tdm_precision net_precision(const tdm_net* net);
// Changes whenever the net's workspace is reallocated or a layer's tile
// changes: a CUDA graph holding a forward of the net is stale after that.
uint64_t net_generation(const tdm_net* net);

// ---- store.cpp: device-resident fragment store ----
struct StoreView {
  const float* keypts;  // k x 3
  const float* desc;    // k x 512
  int32_t k;
  tdm_grid grid;
};
// Reserves (or replaces) entry `key` for k keypoints and returns where to
// write it; the entry is pinned and invisible to readers until committed.
tdm_status store_reserve(tdm_store* st, uint64_t key, uint64_t seed, int32_t k, const tdm_grid* grid, float** keypts,
                         float** desc);
// Ends a write (records the entry's ready event on s); ok = false drops it.
tdm_status store_commit(tdm_store* st, uint64_t key, const tdm_grid* grid, bool ok, cudaStream_t s);
// Pins an entry for reading on stream s (s waits for the entry's writer).
tdm_status store_acquire(tdm_store* st, uint64_t key, StoreView* v, cudaStream_t s);
// Pins an entry against eviction (no stream ordering); false if absent.
bool store_pin(tdm_store* st, uint64_t key);
void store_release(tdm_store* st, uint64_t key);
// Entry present with this keypoint stream and count; `count` updates the
// hit / miss counters and the entry's recency.
bool store_has(tdm_store* st, uint64_t key, uint64_t seed, int32_t k, bool count);
size_t store_entry_bytes(int32_t k);

// ---- pipeline.cu ----
// A pipeline holding only the matching and RANSAC buffers (for pairs of
// already described fragments of up to cfg->max_keypoints keypoints).
tdm_status pipeline_create_match_only(const tdm_pipeline_config* cfg, tdm_pipeline** out);
size_t pipeline_match_bytes(const tdm_pipeline_config* cfg);

}  // namespace tdm

// blocks_tc.cu -- tensor-core (tcgen05) engine for dense k-qubit blocks.
//
// The block acts on every column of the state (one setting of the n-k other
// qubits) as a complex 2^k x 2^k matrix.  Written as a real GEMM,
//   D[m][o] = sum_i A[m][i] * B[o][i],
// A = a tile of 128 state columns, row m holding the 2^k amplitudes of
// column m as interleaved (re, im) reals (i = 2a + c), and B the real form of
// the block matrix: B[2a'+c'][2a+c] = [[Re U, -Im U], [Im U, Re U]][c'][c]
// of U[a'][a].  One tile is an M=128 (columns) x N=2^(k+1) (outputs) x
// K=2^(k+1) (inputs) product on the 5th-generation tensor cores.
//
// Precision: split BF16 x 3.  Every FP32 value x is held as hi = bf16(x),
// lo = bf16(x - hi) (16 significant bits); D = Ahi*Bhi + Ahi*Blo + Alo*Bhi,
// accumulated in FP32 in tensor memory.  The representation error is ~2^-17
// per value and random in sign, so the direction error per block is ~1e-11
// in infidelity.  The tensor cores' FP32 accumulation is not round-to-
// nearest: chaining the K steps shrinks magnitudes by ~1e-6 per block, a
// systematic norm drift (measured: 1 - p(0) = 1.2e-5 after 20 blocks at 30
// qubits).  A unitary block preserves the norm of every column exactly, so
// for unitary blocks the epilogue rescales each output column to the norm of
// its input column (summed in FP32 by the producers), which removes the
// drift; a non-unitary matrix passed to qcs_cuda_apply_block is applied
// without that step.
//
// Kernel structure (persistent, one CTA per SM, 416 threads):
//   warps 0-3   epilogue: tcgen05.ld the accumulator (warp w owns TMEM lanes
//               32w..32w+31 = tile columns), store FP32 results to HBM;
//   warps 4-11  producers: load the tile's amplitudes from HBM, split into
//               bf16 hi/lo, write the 128-byte-swizzled K-major operand tile;
//               the block matrix stays resident in shared memory; loads run
//               one tile ahead in registers, and 2 tiles ahead the tile's
//               contiguous pieces are bulk-prefetched into L2
//   warp 12     TMEM allocation and MMA issue (one thread).
// Operand tiles and TMEM accumulators are double buffered; stages hand over
// through mbarriers.  Every wait is bounded: on expiry the kernel raises a
// device error flag, all roles leave their loops, outstanding MMAs are
// drained and TMEM is freed before exit.
//
// Shared memory (k = 6): 2 stages x (hi + lo) x 32 KB state tiles + 64 KB
// block matrix (hi + lo) + tables, the column-norm ring and the low-mode
// staging = 215 KB.  HBM traffic: one read and one write of the state per
// block; tensor work per amplitude 3 x 8 x 2^k flops.
//
// k = 7 does not fit this layout (its real form alone would take 256 KB):
// k_block_tc7 keeps the real and imaginary parts apart (Tc7, below).
#include <cuda_bf16.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "tcgen05.cuh"

namespace qcs {

constexpr int kTcEpiWarps = 4;
constexpr int kTcProdWarps = 8;
constexpr int kTcMmaWarp = kTcEpiWarps + kTcProdWarps;  // 12
constexpr int kTcThreads = (kTcMmaWarp + 1) * 32;        // 416
constexpr int kTcProdThreads = kTcProdWarps * 32;        // 256
constexpr int kTcEpiThreads = kTcEpiWarps * 32;          // 128
constexpr int kImgSlots = 8;                             // block-matrix upload ring
constexpr int kSqSlots = 4;                              // column-norm ring
constexpr int kEpiPitch = 34;  // floats per staged column (even: 8-byte accesses, 2 wavefronts)

// Memory access modes of the kernel (chosen per block on the host):
//   kColMode   qubit 0 is a column qubit: a warp's 32 columns are adjacent
//              amplitudes, one 8-byte access per amplitude;
//   kPairMode  qubit 0 is block qubit 0: block rows 2b, 2b+1 of a column are
//              adjacent and move as one 16-byte access;
//   kLowMode   the block is exactly qubits 0..k-1: a column is 2^k adjacent
//              amplitudes and the tile one contiguous 128 * 2^k run; a warp
//              loads 512 contiguous bytes per instruction and the epilogue
//              transposes each 32 x 32 result block through shared memory,
//              so that its stores are contiguous too.
constexpr int kColMode = 0, kPairMode = 1, kLowMode = 2;

template <int KA>  // amplitudes per column (2^k)
struct TcShape {
  static constexpr int KD = 2 * KA;              // reals per column: UMMA K extent
  static constexpr int N = 2 * KA;               // reals out per column: UMMA N
  static constexpr int A_BYTES = kTcM * KD * 2;  // one bf16 state operand (hi or lo)
  static constexpr int B_BYTES = N * KD * 2;     // one bf16 matrix operand (hi or lo)
  static constexpr int KSTEPS = KD / 16;         // UMMA K = 16 for bf16
  static constexpr int UNITS = kTcM * KA / 4;    // 4-amplitude units per tile
  static constexpr int UPT = UNITS / kTcProdThreads;
  static constexpr int TMEM_COLS = 2 * N;        // two accumulator stages
  static constexpr int OFF_A = 0;                // [stage][hi,lo][A_BYTES]
  static constexpr int OFF_B = 4 * A_BYTES;      // [hi,lo][B_BYTES]
  static constexpr int OFF_COL = OFF_B + 2 * B_BYTES;
  static constexpr int OFF_BLK = OFF_COL + kTcM * 8;
  static constexpr int OFF_SQ = OFF_BLK + KA * 8;  // float [slot 4][half][column]
  static constexpr int OFF_EPI = OFF_SQ + kSqSlots * 2 * kTcM * 4;  // LOW mode staging
  static constexpr int OFF_BETA = OFF_EPI + kTcEpiWarps * 32 * kEpiPitch * 4;  // float2[KA]
  static constexpr int OFF_BAR = OFF_BETA + KA * 8;
  static constexpr int OFF_MISC = OFF_BAR + 16 * 8;
  static constexpr int SMEM = OFF_MISC + 16 + 1024;  // + slack to align the base to 1 KB
  static constexpr int IMG_BYTES = 2 * B_BYTES;
  static_assert(SMEM <= 232448, "exceeds the 227 KB shared-memory opt-in");
  static_assert(UNITS % kTcProdThreads == 0, "tile units must split over producers");
  static_assert(KD % 64 == 0, "K extent must be whole 128-byte swizzle atoms");
  static_assert(TMEM_COLS == 128 || TMEM_COLS == 256, "TMEM allocation size");
};

// k = 7 (KA = 128): the complex form.  The real form of the matrix would be
// 256 x 256 reals, 256 KB of shared memory in hi + lo, so this kernel keeps
// the real and imaginary parts apart:
//   Re Y = Xr Ur^T - Xi Ui^T,   Im Y = Xr Ui^T + Xi Ur^T,
// A = the tile's real or imaginary parts (M = 128 columns x K = 128
// amplitudes), B = Re U or Im U (N = 128 outputs x K = 128 inputs), the
// minus sign from the instruction descriptor's negate-B bit.  The matrix
// takes 4 x 32 KB (Ur, Ui; hi, lo).  A tile (16384 amplitudes) reaches the
// tensor cores as four K-chunks of 32 amplitudes, each 4 x 8 KB (Xr, Xi;
// hi, lo) in 64-byte swizzle atoms, through two shared-memory stages, so
// that the producers convert one chunk while the tensor cores multiply the
// other.  (One stage of 64-amplitude chunks, the 128-byte layout of the
// other kernel, serialised conversion and MMAs: 0.58-0.63 of HBM at 30
// qubits.)  The accumulators (Re, Im) take 256 TMEM columns per tile,
// double buffered.
struct Tc7 {
  static constexpr int KA = 128;                   // amplitudes per column
  static constexpr int KC = 32;                    // amplitudes per K-chunk
  static constexpr int CHUNKS = KA / KC;           // per tile
  static constexpr int N = KA;                     // UMMA N: outputs of one part
  static constexpr int CH_BYTES = kTcM * KC * 2;   // one bf16 chunk operand
  static constexpr int U_BYTES = N * KA * 2;       // one bf16 matrix operand
  static constexpr int PROD_WARPS = 16;            // producer warps (k_block_tc has 8)
  static constexpr int PROD_THREADS = 32 * PROD_WARPS;
  static constexpr int MMA_WARP = kTcEpiWarps + PROD_WARPS;
  static constexpr int THREADS = 32 * (MMA_WARP + 1);
  static constexpr int SQ_PARTS = PROD_THREADS / kTcM;   // producers per column
  static constexpr int UPT = kTcM * KC / 8 / PROD_THREADS;  // 8-amplitude units per producer
  static constexpr int TMEM_COLS = 512;            // [stage][re, im][N]
  static constexpr int OFF_A = 0;                  // [stage][re hi, re lo, im hi, im lo][CH_BYTES]
  static constexpr int OFF_B = 8 * CH_BYTES;       // [re hi, re lo, im hi, im lo][U_BYTES]
  static constexpr int OFF_COL = OFF_B + 4 * U_BYTES;
  static constexpr int OFF_BLK = OFF_COL + kTcM * 8;
  static constexpr int OFF_SQ = OFF_BLK + KA * 8;  // float [slot 4][part][column]
  static constexpr int OFF_BETA = OFF_SQ + kSqSlots * SQ_PARTS * kTcM * 4;  // float2[KA]
  static constexpr int OFF_EPI = OFF_BETA + KA * 8;  // kLowMode staging
  static constexpr int OFF_BAR = OFF_EPI + kTcEpiWarps * 32 * kEpiPitch * 4;
  static constexpr int OFF_MISC = OFF_BAR + 16 * 8;
  static constexpr int SMEM = OFF_MISC + 16 + 1024;
  static constexpr int IMG_BYTES = 4 * U_BYTES;
  static_assert(SMEM <= 232448, "exceeds the 227 KB shared-memory opt-in");
  static_assert(UPT == 1 && CHUNKS % 2 == 0, "producer shares and stage pairs");
};

// An upload slot: the largest (k = 7) image, then the block's row sums (float2).
constexpr size_t kImgSlotBytes = Tc7::IMG_BYTES + Tc7::KA * 8;

struct TcGeom {
  i64 n_tiles;
  int nfree;
  int nruns;          // prefetch pieces of a tile (at most 128)
  int run_bytes;      // bytes per piece (>= 512 B: the tile holds qubits 0..6)
  int pf_ahead;       // tiles ahead whose pieces are prefetched
  signed char freeq[40];
  i64 col_off[kTcM];  // column m -> offset (bits of m on the column qubits)
  i64 blk_off[128];   // block index a -> offset (bit j of a on qubits[j])
  i64 run_off[128];   // piece j -> offset of its first amplitude
  i64 nib[10][16];    // tile id nibble k with value v -> its part of the tile's offset
};

// Prefetch shape, measured at 30 qubits over six k = 6 block placements
// (mean fraction of measured HBM; two runs agreed within 1 %): 2 tiles ahead
// with whole runs 0.918, with pieces of at most 2^9 amplitudes 0.922, 2^8
// 0.885, 3 tiles ahead 0.85-0.92 depending on the piece.  Whole runs are
// kept: on the 30-qubit brick benchmark pieces of 2^9 measured 1.5 % slower,
// and k = 5 blocks 14 % slower.
// k = 7 tiles are twice as large: 2 tiles ahead measured 0.65 of HBM on
// four placements at 28 qubits (mean), 1 tile ahead 0.79, none 0.71.
static int pf_ahead(int k) { return k == 7 ? 1 : 2; }
static int pf_piece_bits() { return 16; }

// The tile's offset: its id's bits scattered onto the free qubits, four
// bits per table lookup (the index is the same across a warp, so the
// parameter-space reads broadcast).
__device__ __forceinline__ i64 tile_base(i64 tile, const TcGeom &g) {
  i64 b = 0;
  for (int k = 0; 4 * k < g.nfree; k++) b += g.nib[k][(tile >> (4 * k)) & 15];
  return b;
}

// The tiles one CTA processes, in order: tile(it) = start + it * stride for
// it < count, cyclic over the grid (CTA b takes b, b + grid, ...), so that at
// any moment the CTAs work on adjacent tiles.  (A blocked order, each CTA on
// a contiguous range, measured 0.4 % slower on six placements at 30 qubits.)
struct TileWalk {
  i64 start, stride, count;
  __device__ __forceinline__ i64 at(i64 it) const { return start + it * stride; }
};
__device__ __forceinline__ TileWalk tile_walk(const TcGeom &g) {
  const i64 b = blockIdx.x, G = gridDim.x;
  TileWalk w;
  w.start = b;
  w.stride = G;
  w.count = b < g.n_tiles ? (g.n_tiles - b + G - 1) / G : 0;
  return w;
}

// In kColMode and kPairMode a producer thread keeps one column (tile row
// m = p % 128) and consecutive threads take consecutive columns.
// FUSED: the launch may fuse a diffusion in front of the block and/or leave
// the sum of its outputs (the plain instantiation carries neither cost).
template <int KA, int MODE, bool FUSED>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_block_tc(float2 *v, const __grid_constant__ TcGeom g, const uint4 *bimg, int renorm,
               const double *diffuse_sum, double inv_n, ReduceSlot *sum_out, int *err,
               long long wait) {
  using S = TcShape<KA>;
  extern __shared__ uint8_t smem_dyn[];
  const uint32_t raw = smem_u32(smem_dyn);
  uint8_t *smem = smem_dyn + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t *sA = smem + S::OFF_A;
  uint8_t *sB = smem + S::OFF_B;
  i64 *col_off = reinterpret_cast<i64 *>(smem + S::OFF_COL);
  i64 *blk_off = reinterpret_cast<i64 *>(smem + S::OFF_BLK);
  float *colsq = reinterpret_cast<float *>(smem + S::OFF_SQ);
  float *epi = reinterpret_cast<float *>(smem + S::OFF_EPI);
  const uint32_t bar0 = smem_u32(smem + S::OFF_BAR);  // 8-byte barriers:
  // 0,1 a_full[stage]  2,3 mma_done[stage]  4,5 acc_empty[stage]  6 drain
  // 7..10 sq_full[slot]: a tile's column norms are in colsq[slot]
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + S::OFF_MISC);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + S::OFF_MISC + 4);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    mbar_init(bar(0), kTcProdThreads);
    mbar_init(bar(1), kTcProdThreads);
    mbar_init(bar(2), 1);
    mbar_init(bar(3), 1);
    mbar_init(bar(4), kTcEpiThreads);
    mbar_init(bar(5), kTcEpiThreads);
    mbar_init(bar(6), 1);
    for (int k = 0; k < kSqSlots; k++) mbar_init(bar(7 + k), kTcProdThreads);
    *abort_flag = 0;
    fence_barrier_init();
  }
  for (int i = tid; i < kTcM; i += kTcThreads) col_off[i] = g.col_off[i];
  for (int i = tid; i < KA; i += kTcThreads) blk_off[i] = g.blk_off[i];
  {
    uint4 *dst = reinterpret_cast<uint4 *>(sB);
    for (int i = tid; i < S::IMG_BYTES / 16; i += kTcThreads) dst[i] = bimg[i];
  }
  // Diffusion fused in front of the block (diffuse_sum != null): the block
  // reads psi but must act on 2m - psi, m = sum * inv_n; since
  // U (2m 1 - psi) = 2m (U 1) - U psi, the epilogue writes beta - U psi with
  // beta[a] = 2m * (row sum a of U), the row sums following the image.
  float2 *beta = reinterpret_cast<float2 *>(smem + S::OFF_BETA);
  if (FUSED && diffuse_sum) {
    const float tr = (float)(2.0 * (diffuse_sum[0] * inv_n));
    const float ti = (float)(2.0 * (diffuse_sum[1] * inv_n));
    const float2 *rows = reinterpret_cast<const float2 *>(bimg + S::IMG_BYTES / 16);
    for (int i = tid; i < KA; i += kTcThreads) {
      const float2 r = rows[i];
      beta[i] = make_float2(tr * r.x - ti * r.y, tr * r.y + ti * r.x);
    }
  }
  fence_async_shared();  // the block matrix is read by the tensor cores
  if (warp == kTcMmaWarp) {
    tmem_alloc(smem_u32(tmem_slot), S::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp >= kTcEpiWarps && warp < kTcMmaWarp) {
    // ---------------- producers ----------------
    // Stage reuse: the producer of tile it waits for the MMAs of tile it-2.
    // Column-norm slot it % 4 was last read by the epilogue of tile it-4,
    // which finished before the MMAs of tile it-2 could start (they wait for
    // its acc_empty), so the slot is free too.
    // Loads run one tile ahead: a thread holds its share of a tile in two
    // register halves; as soon as a half is converted into the operand, the
    // same registers take the next tile's half, so the next tile's loads are
    // in flight while this tile is converted and while the stage is awaited.
    const int p = tid - kTcEpiThreads;
    constexpr int CPS = 64 / KA;           // kLowMode: columns per 512-byte step
    constexpr int LPC = 32 / CPS;          // kLowMode: lanes per column
    constexpr int STEPS = kTcM / (kTcProdWarps * CPS);
    constexpr int HS = STEPS / 2;          // kLowMode: steps per half
    constexpr int HU = S::UPT / 2;         // other modes: units per half
    const int pw = p >> 5;
    const int r2 = 2 * (lane % LPC);       // kLowMode: first of the lane's two rows
    const int mc = p & (kTcM - 1);         // other modes: the thread's column
    float4 xl[2][HS];                      // kLowMode data, by half
    float2 xc[2][HU][4];                   // other modes' data, by half
    auto load_half = [&](i64 base, int h) {
      if constexpr (MODE == kLowMode) {
#pragma unroll
        for (int i = 0; i < HS; i++) {
          const int m = (pw * STEPS + h * HS + i) * CPS + lane / LPC;
          xl[h][i] = *reinterpret_cast<const float4 *>(v + base + col_off[m] + r2);
        }
      } else {
        const float2 *src = v + base + col_off[mc];
#pragma unroll
        for (int i = 0; i < HU; i++) {
          const int j = (p >> 7) + 2 * (h * HU + i);  // unit: block rows 4j .. 4j+3
          if constexpr (MODE == kPairMode) {
            const float4 a = *reinterpret_cast<const float4 *>(src + blk_off[4 * j]);
            const float4 b = *reinterpret_cast<const float4 *>(src + blk_off[4 * j + 2]);
            xc[h][i][0] = make_float2(a.x, a.y);
            xc[h][i][1] = make_float2(a.z, a.w);
            xc[h][i][2] = make_float2(b.x, b.y);
            xc[h][i][3] = make_float2(b.z, b.w);
          } else {
#pragma unroll
            for (int e = 0; e < 4; e++) xc[h][i][e] = src[blk_off[4 * j + e]];
          }
        }
      }
    };
    float part[STEPS];  // kLowMode: per-step partial norms; [0]: other modes
    auto convert_half = [&](int h, uint8_t *ahi, uint8_t *alo) {
      if constexpr (MODE == kLowMode) {
#pragma unroll
        for (int i = 0; i < HS; i++) {
          const float4 x = xl[h][i];
          const int m = (pw * STEPS + h * HS + i) * CPS + lane / LPC;
          __nv_bfloat162 h0 = __floats2bfloat162_rn(x.x, x.y);
          __nv_bfloat162 h1 = __floats2bfloat162_rn(x.z, x.w);
          const float2 f0 = __bfloat1622float2(h0), f1 = __bfloat1622float2(h1);
          __nv_bfloat162 l0 = __floats2bfloat162_rn(x.x - f0.x, x.y - f0.y);
          __nv_bfloat162 l1 = __floats2bfloat162_rn(x.z - f1.x, x.w - f1.y);
          const int off = sw128_offset(m, 2 * r2, kTcM);
          *reinterpret_cast<uint2 *>(ahi + off) =
              make_uint2(*reinterpret_cast<uint32_t *>(&h0), *reinterpret_cast<uint32_t *>(&h1));
          *reinterpret_cast<uint2 *>(alo + off) =
              make_uint2(*reinterpret_cast<uint32_t *>(&l0), *reinterpret_cast<uint32_t *>(&l1));
          part[h * HS + i] = x.x * x.x + x.y * x.y + x.z * x.z + x.w * x.w;
        }
      } else {
#pragma unroll
        for (int i = 0; i < HU; i++) {
          const int j = (p >> 7) + 2 * (h * HU + i);
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const float2 x = xc[h][i][e];
            __nv_bfloat162 hb = __floats2bfloat162_rn(x.x, x.y);
            float2 hf = __bfloat1622float2(hb);
            __nv_bfloat162 lb = __floats2bfloat162_rn(x.x - hf.x, x.y - hf.y);
            hw[e] = *reinterpret_cast<uint32_t *>(&hb);
            lw[e] = *reinterpret_cast<uint32_t *>(&lb);
            part[0] += x.x * x.x + x.y * x.y;
          }
          const int off = sw128_offset(mc, 8 * j, kTcM);
          *reinterpret_cast<uint4 *>(ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4 *>(alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
      }
    };
    const TileWalk w = tile_walk(g);
    if (w.count > 0) {
      const i64 base = tile_base(w.at(0), g);
      load_half(base, 0);
      load_half(base, 1);
    }
    for (int it = 0; it < w.count; ++it) {
      const int stage = it & 1;
      const bool more = it + 1 < w.count;
      const i64 nbase = more ? tile_base(w.at(it + 1), g) : 0;
      // the pieces of the tile pf_ahead ahead go to L2 now, so that the
      // register loads issued for later tiles find them there
      if (p < g.nruns && it + g.pf_ahead < w.count)  // nruns <= 128 < 256 producers
        prefetch_l2(v + tile_base(w.at(it + g.pf_ahead), g) + g.run_off[p],
                    (uint32_t)g.run_bytes);
      // in low mode every lane of a warp takes the same decision: the norm
      // exchange below is a full-warp shuffle
      if (it >= 2) {
        bool ok = wait_bar(bar(2 + stage), ((it - 2) >> 1) & 1, abort_flag, err, 1, wait);
        if (MODE == kLowMode) ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
      }
      uint8_t *ahi = sA + (2 * stage) * S::A_BYTES;
      uint8_t *alo = ahi + S::A_BYTES;
      float *sq = colsq + (it % kSqSlots) * 2 * kTcM;
      part[0] = 0.f;
      convert_half(0, ahi, alo);
      if (more) load_half(nbase, 0);
      convert_half(1, ahi, alo);
      if (more) load_half(nbase, 1);
      if constexpr (MODE == kLowMode) {
        // Column norms: part[i] of lane l belongs to the warp's column
        // i * CPS + l / LPC.  A reduce-scatter over the LPC lanes of each
        // column (fixed order, deterministic): after the step with offset o
        // a lane keeps the half of its values selected by (l & o), so lane
        // bits 1.. select the surviving column; a last exchange with the
        // neighbour lane completes the sum.
        constexpr int LOG_STEPS = STEPS == 16 ? 4 : 3;
        static_assert(STEPS == (1 << LOG_STEPS) && STEPS * 2 == LPC, "reduce-scatter shape");
#pragma unroll
        for (int st = 0; st < LOG_STEPS; st++) {
          const int o = LPC >> (st + 1);
          const int half = STEPS >> (st + 1);
          const bool up = (lane & o) != 0;
#pragma unroll
          for (int j = 0; j < half; j++) {
            const float send = up ? part[j] : part[half + j];
            const float keep = up ? part[half + j] : part[j];
            part[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
          }
        }
        part[0] += __shfl_xor_sync(0xffffffffu, part[0], 1);
        if ((lane & 1) == 0) {
          const int i_sel = (lane % LPC) >> 1;
          const int m = (pw * STEPS + i_sel) * CPS + lane / LPC;
          sq[m] = part[0];
          sq[kTcM + m] = 0.f;
        }
      } else {
        // threads p and p + 128 hold the two halves of column mc's norm
        sq[(p >> 7) * kTcM + mc] = part[0];
      }
      fence_async_shared();
      mbar_arrive(bar(stage));
      mbar_arrive(bar(7 + it % kSqSlots));
    }
  } else if (warp == kTcMmaWarp) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(kTcM, S::N);
      const uint32_t a0 = smem_u32(sA), b_hi = smem_u32(sB), b_lo = b_hi + S::B_BYTES;
      const TileWalk w = tile_walk(g);
      for (int it = 0; it < w.count; ++it) {
        const int stage = it & 1;
        if (!wait_bar(bar(stage), (it >> 1) & 1, abort_flag, err, 2, wait)) break;
        if (it >= 2 && !wait_bar(bar(4 + stage), ((it - 2) >> 1) & 1, abort_flag, err, 3, wait))
          break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(stage * S::N);
        const uint32_t a_hi = a0 + (uint32_t)(2 * stage * S::A_BYTES);
        const uint32_t a_lo = a_hi + S::A_BYTES;
#pragma unroll
        for (int s = 0; s < S::KSTEPS; s++) {
          const uint32_t ka = (uint32_t)((s >> 2) * (kTcM * 128) + (s & 3) * 32);
          const uint32_t kb = (uint32_t)((s >> 2) * (S::N * 128) + (s & 3) * 32);
          umma_bf16(d, sw128_desc(a_hi + ka), sw128_desc(b_hi + kb), idesc, s > 0 ? 1u : 0u);
          umma_bf16(d, sw128_desc(a_hi + ka), sw128_desc(b_lo + kb), idesc, 1u);
          umma_bf16(d, sw128_desc(a_lo + ka), sw128_desc(b_hi + kb), idesc, 1u);
        }
        umma_commit(bar(2 + stage));
      }
      // every MMA issued above must finish before TMEM is released
      umma_commit(bar(6));
      long long t0 = clock64();
      while (!mbar_try_wait(bar(6), 0)) {
        if (clock64() - t0 > kWaitCycles) {
          atomicExch(err, 4);
          break;
        }
      }
    }
    __syncwarp();
  } else {
    // ---------------- epilogue ----------------
    const int m = tid;  // TMEM lane = tile column
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
    const TileWalk w = tile_walk(g);
    double sum_re = 0.0, sum_im = 0.0;  // sum of this thread's outputs (sum_out)
    // Output values of result block c (rows 16c .. 16c+15, re/im
    // interleaved): the norm-restoring scale, then the fused diffusion's
    // affine term; their FP32 sum feeds sum_out.
    auto finish = [&](float *acc, int c, float scale) {
      if constexpr (!FUSED) {
#pragma unroll
        for (int q = 0; q < 32; q++) acc[q] *= scale;
      } else {
        float pr = 0.f, pi = 0.f;
#pragma unroll
        for (int q = 0; q < 16; q++) {
          float re = acc[2 * q] * scale, im = acc[2 * q + 1] * scale;
          if (diffuse_sum) {
            const float2 b = beta[16 * c + q];
            re = b.x - re;
            im = b.y - im;
          }
          acc[2 * q] = re;
          acc[2 * q + 1] = im;
          pr += re;
          pi += im;
        }
        if (sum_out) {
          sum_re += (double)pr;
          sum_im += (double)pi;
        }
      }
    };
    for (int it = 0; it < w.count; ++it) {
      const i64 tile = w.at(it);
      const int stage = it & 1;
      bool ok = wait_bar(bar(2 + stage), (it >> 1) & 1, abort_flag, err, 5, wait);
      // this tile's column norms; slot it % 4 cannot be refilled before this
      // epilogue arrives on acc_empty, so its phase is unambiguous
      ok = ok && wait_bar(bar(7 + it % kSqSlots), (it / kSqSlots) & 1, abort_flag, err, 6, wait);
      if (!__all_sync(0xffffffffu, ok)) break;  // the warp's TMEM loads are .sync.aligned
      tc_fence_after();
      const uint32_t tb = tmem + lane_addr + (uint32_t)(stage * S::N);
      float scale = 1.f;
      // TMEM is read 64 columns per instruction: each tcgen05.ld waits for
      // its data, and the epilogue is the slower side of the pipeline when
      // the loads are contiguous
      if (renorm) {
        float out = 0.f;
#pragma unroll 1
        for (int cc = 0; cc < S::N / 64; cc++) {
          float acc[64];
          tmem_ld64(tb + 64 * cc, acc);
#pragma unroll
          for (int q = 0; q < 64; q++) out += acc[q] * acc[q];
        }
        const float *sq = colsq + (it % kSqSlots) * 2 * kTcM;
        const float in = sq[m] + sq[kTcM + m];
        if (out > 0.f) scale = sqrtf(in / out);
      }
      const i64 base = tile_base(tile, g);
      if constexpr (MODE == kLowMode) {
        // Result block c of this warp: 32 columns x 32 reals (rows 16c ..
        // 16c+15), transposed through shared memory so that each store
        // instruction writes one column's 16 adjacent amplitudes (128 B).
        // Staged as float2: lane m writes its column's 16 amplitudes in row m;
        // then lanes 0-15 store column j and lanes 16-31 column j+1, one
        // amplitude each, two full 128-byte lines per instruction.
        float *buf = epi + warp * 32 * kEpiPitch;
        const int half = lane >> 4, row = lane & 15;
#pragma unroll 1
        for (int cc = 0; cc < S::N / 64; cc++) {
          float acc[64];
          tmem_ld64(tb + 64 * cc, acc);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const int c = 2 * cc + h;
            float *a = acc + 32 * h;
            finish(a, c, scale);
#pragma unroll
            for (int q = 0; q < 16; q++)
              *reinterpret_cast<float2 *>(buf + lane * kEpiPitch + 2 * q) =
                  make_float2(a[2 * q], a[2 * q + 1]);
            __syncwarp();
#pragma unroll 4
            for (int j = 0; j < 32; j += 2) {
              const float2 val =
                  *reinterpret_cast<const float2 *>(buf + (j + half) * kEpiPitch + 2 * row);
              v[base + col_off[warp * 32 + j + half] + 16 * c + row] = val;
            }
            __syncwarp();
          }
        }
      } else {
      float2 *dst = v + base + col_off[m];
#pragma unroll 1
      for (int cc = 0; cc < S::N / 64; cc++) {
        float acc[64];
        tmem_ld64(tb + 64 * cc, acc);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = 2 * cc + h;
          float *a = acc + 32 * h;
          finish(a, c, scale);
          if constexpr (MODE == kPairMode) {
#pragma unroll
            for (int q = 0; q < 8; q++)
              *reinterpret_cast<float4 *>(dst + blk_off[16 * c + 2 * q]) =
                  make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
          } else {
#pragma unroll
            for (int q = 0; q < 16; q++)
              dst[blk_off[16 * c + q]] = make_float2(a[2 * q], a[2 * q + 1]);
          }
        }
      }
      }
      tc_fence_before();
      mbar_arrive(bar(4 + stage));
    }
    if (FUSED && sum_out) {  // one slot per epilogue warp, combined in order afterwards
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum_re += __shfl_xor_sync(0xffffffffu, sum_re, o);
        sum_im += __shfl_xor_sync(0xffffffffu, sum_im, o);
      }
      if (lane == 0) {
        ReduceSlot r;
        r.a = sum_re;
        r.b = sum_im;
        r.c = 0.0;
        r.d = 0.0;
        sum_out[blockIdx.x * kTcEpiWarps + warp] = r;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kTcMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem, S::TMEM_COLS);
  }
}

// k = 7 (the complex form, Tc7).  Same roles, waits and fused epilogue as
// k_block_tc, with 16 producer warps instead of 8 (672 threads, 80
// registers a thread); what differs is the operand layout and the chunked
// pipeline:
//   producers  convert chunk q (tile q / 4, amplitudes 32 (q % 4) ..) into
//              stage q % 2 once the MMAs of chunk q - 2 are done, holding
//              chunks q + 1 and q + 2 in flight in registers meanwhile;
//   MMA        12 products per 16-amplitude K-step (Re, Im x 3 split terms x
//              2 parts), committing a stage back after every chunk and the
//              accumulator pair after a tile's last chunk;
//   epilogue   reads Re and Im of 16 outputs at a time, both loads under
//              one completion wait.
// In kLowMode (the block is qubits 0..6) a column is 128 adjacent
// amplitudes: a producer lane converts 4 adjacent amplitudes of a column (two
// 16-byte loads, one 8-byte store per operand), so a warp's load pair reads
// 256 contiguous bytes of each of 4 columns; the epilogue transposes 32 x 16
// results through shared memory, as in k_block_tc.
// The other modes load and store the state evict-first (ld/st .cs): each
// line is read once and written once, and so marked it leaves L2 before the
// tile the bulk prefetch brought in ahead.  A block on high qubits spreads a
// tile over 128 far-apart runs, where plain accesses evicted part of the
// prefetched tile (at 26 qubits, qubits 19..25 read 9 % more DRAM bytes than
// the state, qubits 7..13 2 %).  At 30 qubits the hint measured 3-9 % faster
// on placements above qubit 12, and no change on qubits 7..13; in kLowMode
// and in k_block_tc it measured no faster or slower, so those keep plain
// accesses.
template <int MODE, bool FUSED>
__global__ void __launch_bounds__(Tc7::THREADS, 1)
    k_block_tc7(float2 *v, const __grid_constant__ TcGeom g, const uint4 *bimg, int renorm,
                const double *diffuse_sum, double inv_n, ReduceSlot *sum_out, int *err,
                long long wait) {
  using S = Tc7;
  extern __shared__ uint8_t smem_dyn[];
  const uint32_t raw = smem_u32(smem_dyn);
  uint8_t *smem = smem_dyn + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t *sA = smem + S::OFF_A;
  uint8_t *sB = smem + S::OFF_B;
  i64 *col_off = reinterpret_cast<i64 *>(smem + S::OFF_COL);
  i64 *blk_off = reinterpret_cast<i64 *>(smem + S::OFF_BLK);
  float *colsq = reinterpret_cast<float *>(smem + S::OFF_SQ);
  float *epi = reinterpret_cast<float *>(smem + S::OFF_EPI);
  const uint32_t bar0 = smem_u32(smem + S::OFF_BAR);  // 8-byte barriers:
  // 0,1 chunk_full[stage]  2,3 chunk_free[stage]  4,5 acc_full[acc]
  // 6,7 acc_empty[acc]  8 drain  9..12 sq_full[slot]: a tile's column norms
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + S::OFF_MISC);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + S::OFF_MISC + 4);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    mbar_init(bar(0), S::PROD_THREADS);
    mbar_init(bar(1), S::PROD_THREADS);
    mbar_init(bar(2), 1);
    mbar_init(bar(3), 1);
    mbar_init(bar(4), 1);
    mbar_init(bar(5), 1);
    mbar_init(bar(6), kTcEpiThreads);
    mbar_init(bar(7), kTcEpiThreads);
    mbar_init(bar(8), 1);
    for (int k = 0; k < kSqSlots; k++) mbar_init(bar(9 + k), S::PROD_THREADS);
    *abort_flag = 0;
    fence_barrier_init();
  }
  for (int i = tid; i < kTcM; i += S::THREADS) col_off[i] = g.col_off[i];
  for (int i = tid; i < S::KA; i += S::THREADS) blk_off[i] = g.blk_off[i];
  {
    uint4 *dst = reinterpret_cast<uint4 *>(sB);
    for (int i = tid; i < S::IMG_BYTES / 16; i += S::THREADS) dst[i] = bimg[i];
  }
  float2 *beta = reinterpret_cast<float2 *>(smem + S::OFF_BETA);
  if (FUSED && diffuse_sum) {  // as in k_block_tc: beta[a] = 2m * (row sum a of U)
    const float tr = (float)(2.0 * (diffuse_sum[0] * inv_n));
    const float ti = (float)(2.0 * (diffuse_sum[1] * inv_n));
    const float2 *rows = reinterpret_cast<const float2 *>(bimg + S::IMG_BYTES / 16);
    for (int i = tid; i < S::KA; i += S::THREADS) {
      const float2 r = rows[i];
      beta[i] = make_float2(tr * r.x - ti * r.y, tr * r.y + ti * r.x);
    }
  }
  fence_async_shared();
  if (warp == S::MMA_WARP) {
    tmem_alloc(smem_u32(tmem_slot), S::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp >= kTcEpiWarps && warp < S::MMA_WARP) {
    // ---------------- producers ----------------
    // Thread p keeps column mc = p % 128; of a chunk's 4 units of 8
    // amplitudes it takes units p / 128 and p / 128 + 2.  Chunk q's
    // amplitudes are loaded into register set q % 2 while chunk q - 2 is
    // converted out of it, two chunks ahead of their conversion.  Column-norm
    // slot it % 4 is free when tile it's last chunk is converted: the MMAs of
    // its earlier chunks ran, so the epilogue of tile it - 2 (and with it
    // that of tile it - 4, the slot's last reader) is done.
    const int p = tid - kTcEpiThreads;
    const int mc = p & (kTcM - 1);
    const int pw = p >> 5;
    // kLowMode: a warp instruction covers 4 columns, 8 lanes a column and 4
    // adjacent amplitudes a lane (32 bytes: two 16-byte loads)
    constexpr int LCOLS = 4;
    constexpr int LSTEPS = kTcM / (LCOLS * S::PROD_WARPS);  // 4-column steps per chunk
    float2 xc[2][S::UPT][8];   // other modes: [chunk parity][unit][amplitude]
    float4 xl[2][LSTEPS][2];   // kLowMode: [chunk parity][step][amplitudes 0-1, 2-3]
    float partl[LSTEPS];       // kLowMode: per-step column norms over a tile
    const TileWalk w = tile_walk(g);
    const i64 nq = (i64)S::CHUNKS * w.count;  // chunks, an even number
    i64 load_tile = -1, load_base = 0;  // the tile base, computed once per tile
    auto load_chunk = [&](auto bc, i64 q) {
      constexpr int b = decltype(bc)::value;
      if (q / S::CHUNKS != load_tile) {
        load_tile = q / S::CHUNKS;
        load_base = tile_base(w.at(load_tile), g);
      }
      const i64 base = load_base;
      const int c = (int)(q % S::CHUNKS);
      if constexpr (MODE == kLowMode) {
#pragma unroll
        for (int i = 0; i < LSTEPS; i++) {
          const int m = pw * LCOLS * LSTEPS + LCOLS * i + (lane >> 3);
          const float4 *src = reinterpret_cast<const float4 *>(v + base + col_off[m] +
                                                               c * S::KC + 4 * (lane & 7));
          xl[b][i][0] = src[0];
          xl[b][i][1] = src[1];
        }
      } else {
        const float2 *src = v + base + col_off[mc];
#pragma unroll
        for (int i = 0; i < S::UPT; i++) {
          const int a = c * S::KC + 8 * ((p >> 7) + S::SQ_PARTS * i);
          if constexpr (MODE == kPairMode) {
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
              const float4 t = __ldcs(reinterpret_cast<const float4 *>(src + blk_off[a + e]));
              xc[b][i][e] = make_float2(t.x, t.y);
              xc[b][i][e + 1] = make_float2(t.z, t.w);
            }
          } else {
#pragma unroll
            for (int e = 0; e < 8; e++) xc[b][i][e] = __ldcs(src + blk_off[a + e]);
          }
        }
      }
    };
    float part = 0.f;
    // hi and lo of two amplitudes' real and imaginary parts
    auto split2 = [&](float2 x0, float2 x1, uint32_t *wd) {
      const __nv_bfloat162 rh = __floats2bfloat162_rn(x0.x, x1.x);
      const __nv_bfloat162 ih = __floats2bfloat162_rn(x0.y, x1.y);
      const float2 rf = __bfloat1622float2(rh), imf = __bfloat1622float2(ih);
      const __nv_bfloat162 rl = __floats2bfloat162_rn(x0.x - rf.x, x1.x - rf.y);
      const __nv_bfloat162 il = __floats2bfloat162_rn(x0.y - imf.x, x1.y - imf.y);
      wd[0] = *reinterpret_cast<const uint32_t *>(&rh);
      wd[1] = *reinterpret_cast<const uint32_t *>(&rl);
      wd[2] = *reinterpret_cast<const uint32_t *>(&ih);
      wd[3] = *reinterpret_cast<const uint32_t *>(&il);
      return x0.x * x0.x + x0.y * x0.y + x1.x * x1.x + x1.y * x1.y;
    };
    auto convert_chunk = [&](auto bc) {
      constexpr int b = decltype(bc)::value;
      uint8_t *st = sA + b * 4 * S::CH_BYTES;
      if constexpr (MODE == kLowMode) {
#pragma unroll
        for (int i = 0; i < LSTEPS; i++) {
          const float4 x0 = xl[b][i][0], x1 = xl[b][i][1];
          const int m = pw * LCOLS * LSTEPS + LCOLS * i + (lane >> 3);
          uint32_t w0[4], w1[4];
          partl[i] += split2(make_float2(x0.x, x0.y), make_float2(x0.z, x0.w), w0);
          partl[i] += split2(make_float2(x1.x, x1.y), make_float2(x1.z, x1.w), w1);
          // 4 bf16 = 8 bytes inside one 16-byte swizzle chunk
          const int off = sw64_offset(m, 4 * (lane & 7));
#pragma unroll
          for (int o = 0; o < 4; o++)
            *reinterpret_cast<uint2 *>(st + o * S::CH_BYTES + off) = make_uint2(w0[o], w1[o]);
        }
      } else {
#pragma unroll
        for (int i = 0; i < S::UPT; i++) {
          const int j = (p >> 7) + S::SQ_PARTS * i;
          uint32_t wd[4][4];  // [re hi, re lo, im hi, im lo][pair of amplitudes]
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            uint32_t t[4];
            part += split2(xc[b][i][e], xc[b][i][e + 1], t);
#pragma unroll
            for (int o = 0; o < 4; o++) wd[o][e / 2] = t[o];
          }
          const int off = sw64_offset(mc, 8 * j);
#pragma unroll
          for (int o = 0; o < 4; o++)
            *reinterpret_cast<uint4 *>(st + o * S::CH_BYTES + off) =
                make_uint4(wd[o][0], wd[o][1], wd[o][2], wd[o][3]);
        }
      }
    };
    // the tile's column norms into slot it % 4: kLowMode sums each column's
    // 8 lanes (fixed order); otherwise threads p and p + 128 hold the halves
    auto store_norms = [&](i64 it) {
      float *sq = colsq + (it % kSqSlots) * S::SQ_PARTS * kTcM;
      if constexpr (MODE == kLowMode) {
#pragma unroll
        for (int i = 0; i < LSTEPS; i++) {
          float x = partl[i];
#pragma unroll
          for (int o = 1; o < 8; o <<= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          if ((lane & 7) == 0) {
            const int m = pw * LCOLS * LSTEPS + LCOLS * i + (lane >> 3);
            sq[m] = x;
#pragma unroll
            for (int h = 1; h < S::SQ_PARTS; h++) sq[h * kTcM + m] = 0.f;
          }
        }
      } else {
        sq[(p >> 7) * kTcM + mc] = part;  // part p / 128 of column mc's norm
      }
    };
    // one chunk: false when the CTA is aborting
    auto step = [&](auto bc, i64 q) -> bool {
      constexpr int b = decltype(bc)::value;
      const i64 it = q / S::CHUNKS;
      const int c = (int)(q % S::CHUNKS);
      if (c == 0 && p < g.nruns && it + g.pf_ahead < w.count)
        prefetch_l2(v + tile_base(w.at(it + g.pf_ahead), g) + g.run_off[p],
                    (uint32_t)g.run_bytes);
      // stage b is free once the MMAs of chunk q - 2 are done
      if (q >= 2) {
        bool ok = wait_bar(bar(2 + b), (uint32_t)(((q - 2) >> 1) & 1), abort_flag, err, 1, wait);
        if (MODE == kLowMode) ok = __all_sync(0xffffffffu, ok);  // low-mode norm shuffles
        if (!ok) return false;
      }
      if (c == 0) {
        part = 0.f;
#pragma unroll
        for (int i = 0; i < LSTEPS; i++) partl[i] = 0.f;
      }
      convert_chunk(bc);
      if (q + 2 < nq) load_chunk(bc, q + 2);
      if (c == S::CHUNKS - 1) store_norms(it);
      fence_async_shared();
      mbar_arrive(bar(b));
      if (c == S::CHUNKS - 1) mbar_arrive(bar(9 + (int)(it % kSqSlots)));
      return true;
    };
    const std::integral_constant<int, 0> b0{};
    const std::integral_constant<int, 1> b1{};
    if (nq > 0) {
      load_chunk(b0, 0);
      load_chunk(b1, 1);
    }
    for (i64 q = 0; q < nq; q += 2)
      if (!step(b0, q) || !step(b1, q + 1)) break;
  } else if (warp == S::MMA_WARP) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(kTcM, S::N);
      constexpr uint32_t idesc_neg = idesc | (1u << 14);  // negate B
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
      const TileWalk w = tile_walk(g);
      bool ok = true;
      for (i64 it = 0; ok && it < w.count; ++it) {
        const int acc_st = (int)(it & 1);
        if (it >= 2 &&
            !wait_bar(bar(6 + acc_st), (uint32_t)(((it - 2) >> 1) & 1), abort_flag, err, 3, wait))
          break;
        const uint32_t dr = tmem + (uint32_t)(acc_st * 2 * S::N), di = dr + (uint32_t)S::N;
        for (int c = 0; c < S::CHUNKS; c++) {
          const i64 q = it * S::CHUNKS + c;
          const int b = (int)(q & 1);
          if (!wait_bar(bar(b), (uint32_t)((q >> 1) & 1), abort_flag, err, 2, wait)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t as = a0 + (uint32_t)(b * 4 * S::CH_BYTES);
#pragma unroll
          for (int s = 0; s < S::KC / 16; s++) {
            const int kk = c * S::KC + 16 * s;  // K index into the matrix
            const uint32_t ka = (uint32_t)(s * 32);
            const uint32_t kb = (uint32_t)((kk >> 6) * (S::N * 128) + (kk & 63) * 2);
            const uint64_t xrh = sw64_desc(as + 0 * S::CH_BYTES + ka);
            const uint64_t xrl = sw64_desc(as + 1 * S::CH_BYTES + ka);
            const uint64_t xih = sw64_desc(as + 2 * S::CH_BYTES + ka);
            const uint64_t xil = sw64_desc(as + 3 * S::CH_BYTES + ka);
            const uint64_t urh = sw128_desc(b0 + 0 * S::U_BYTES + kb);
            const uint64_t url = sw128_desc(b0 + 1 * S::U_BYTES + kb);
            const uint64_t uih = sw128_desc(b0 + 2 * S::U_BYTES + kb);
            const uint64_t uil = sw128_desc(b0 + 3 * S::U_BYTES + kb);
            const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
            umma_bf16(dr, xrh, urh, idesc, acc);  // Re += Xr Ur
            umma_bf16(dr, xrh, url, idesc, 1u);
            umma_bf16(dr, xrl, urh, idesc, 1u);
            umma_bf16(dr, xih, uih, idesc_neg, 1u);  // Re -= Xi Ui
            umma_bf16(dr, xih, uil, idesc_neg, 1u);
            umma_bf16(dr, xil, uih, idesc_neg, 1u);
            umma_bf16(di, xrh, uih, idesc, acc);  // Im += Xr Ui
            umma_bf16(di, xrh, uil, idesc, 1u);
            umma_bf16(di, xrl, uih, idesc, 1u);
            umma_bf16(di, xih, urh, idesc, 1u);  // Im += Xi Ur
            umma_bf16(di, xih, url, idesc, 1u);
            umma_bf16(di, xil, urh, idesc, 1u);
          }
          umma_commit(bar(2 + b));
        }
        if (ok) umma_commit(bar(4 + acc_st));
      }
      umma_commit(bar(8));
      long long t0 = clock64();
      while (!mbar_try_wait(bar(8), 0)) {
        if (clock64() - t0 > kWaitCycles) {
          atomicExch(err, 4);
          break;
        }
      }
    }
    __syncwarp();
  } else {
    // ---------------- epilogue ----------------
    const int m = tid;  // TMEM lane = tile column
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
    const TileWalk w = tile_walk(g);
    double sum_re = 0.0, sum_im = 0.0;
    for (i64 it = 0; it < w.count; ++it) {
      const i64 tile = w.at(it);
      const int acc_st = (int)(it & 1);
      bool ok = wait_bar(bar(4 + acc_st), (uint32_t)((it >> 1) & 1), abort_flag, err, 5, wait);
      ok = ok && wait_bar(bar(9 + (int)(it % kSqSlots)), (uint32_t)((it / kSqSlots) & 1),
                          abort_flag, err, 6, wait);
      if (!__all_sync(0xffffffffu, ok)) break;  // the warp's TMEM loads are .sync.aligned
      tc_fence_after();
      const uint32_t tr = tmem + lane_addr + (uint32_t)(acc_st * 2 * S::N);
      const uint32_t ti = tr + (uint32_t)S::N;
      float scale = 1.f;
      if (renorm) {
        float out = 0.f;
#pragma unroll 1
        for (int cc = 0; cc < 2 * S::N / 32; cc++) {  // Re then Im: adjacent columns
          float acc[32];  // 32 columns a wait: 21 warps leave 80 registers a thread
          tmem_ld16x2(tr + 32 * cc, tr + 32 * cc + 16, acc, acc + 16);
#pragma unroll
          for (int q = 0; q < 32; q++) out += acc[q] * acc[q];
        }
        const float *sq = colsq + (it % kSqSlots) * S::SQ_PARTS * kTcM;
        float in = 0.f;
#pragma unroll
        for (int h = 0; h < S::SQ_PARTS; h++) in += sq[h * kTcM + m];
        if (out > 0.f) scale = sqrtf(in / out);
      }
      const i64 tbase = tile_base(tile, g);
      float2 *dst = v + tbase + col_off[m];
      // 16 outputs at a time: 21 warps leave 80 registers a thread
#pragma unroll 1
      for (int gq = 0; gq < S::N / 16; gq++) {
        float re[16], im[16];
        tmem_ld16x2(tr + 16 * gq, ti + 16 * gq, re, im);
        float pr = 0.f, pi = 0.f;
#pragma unroll
        for (int q = 0; q < 16; q++) {
          re[q] *= scale;
          im[q] *= scale;
          if constexpr (FUSED) {
            if (diffuse_sum) {
              const float2 b = beta[16 * gq + q];
              re[q] = b.x - re[q];
              im[q] = b.y - im[q];
            }
            pr += re[q];
            pi += im[q];
          }
        }
        if constexpr (FUSED) {
          if (sum_out) {
            sum_re += (double)pr;
            sum_im += (double)pi;
          }
        }
        if constexpr (MODE == kLowMode) {
          // 32 columns x 16 outputs through the warp's staging rows; then
          // lanes 0-15 store column j and lanes 16-31 column j + 1, one
          // amplitude each: two full 128-byte lines per instruction
          float *buf = epi + warp * 32 * kEpiPitch;
          const int half = lane >> 4, row = lane & 15;
#pragma unroll
          for (int q = 0; q < 16; q++)
            *reinterpret_cast<float2 *>(buf + lane * kEpiPitch + 2 * q) = make_float2(re[q], im[q]);
          __syncwarp();
#pragma unroll 4
          for (int j = 0; j < 32; j += 2) {
            const float2 val =
                *reinterpret_cast<const float2 *>(buf + (j + half) * kEpiPitch + 2 * row);
            v[tbase + col_off[warp * 32 + j + half] + 16 * gq + row] = val;
          }
          __syncwarp();
        } else if constexpr (MODE == kPairMode) {
#pragma unroll
          for (int q = 0; q < 16; q += 2)
            __stcs(reinterpret_cast<float4 *>(dst + blk_off[16 * gq + q]),
                   make_float4(re[q], im[q], re[q + 1], im[q + 1]));
        } else {
#pragma unroll
          for (int q = 0; q < 16; q++) __stcs(dst + blk_off[16 * gq + q], make_float2(re[q], im[q]));
        }
      }
      tc_fence_before();
      mbar_arrive(bar(6 + acc_st));
    }
    if (FUSED && sum_out) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sum_re += __shfl_xor_sync(0xffffffffu, sum_re, o);
        sum_im += __shfl_xor_sync(0xffffffffu, sum_im, o);
      }
      if (lane == 0) {
        ReduceSlot r;
        r.a = sum_re;
        r.b = sum_im;
        r.c = 0.0;
        r.d = 0.0;
        sum_out[blockIdx.x * kTcEpiWarps + warp] = r;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == S::MMA_WARP) {
    tc_fence_after();
    tmem_dealloc(tmem, S::TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct TcRing {
  uint8_t *host = nullptr;  // pinned, kImgSlots images
  uint8_t *dev = nullptr;
  cudaEvent_t done[kImgSlots] = {};
  int next = 0;
  int *d_err = nullptr;
};

static int ring_init(qcs_cuda_state *s) {
  if (s->tc) return QCS_CUDA_OK;
  TcRing *r = new TcRing();
  const size_t bytes = (size_t)kImgSlots * kImgSlotBytes;
  int rc = check_cuda(cudaMallocHost((void **)&r->host, bytes), "cudaMallocHost(block images)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&r->dev, bytes), "cudaMalloc(block images)");
  for (int i = 0; !rc && i < kImgSlots; i++)
    rc = check_cuda(cudaEventCreateWithFlags(&r->done[i], cudaEventDisableTiming), "cudaEventCreate");
  if (rc) {
    tc_release(r);
    return rc;
  }
  s->tc = r;
  return QCS_CUDA_OK;
}

void tc_release(TcRing *r) {
  if (!r) return;
  for (int i = 0; i < kImgSlots; i++)
    if (r->done[i]) cudaEventDestroy(r->done[i]);
  if (r->host) cudaFreeHost(r->host);
  if (r->dev) cudaFree(r->dev);
  delete r;
}

bool tc_supported(const qcs_cuda_state *s, int k) {
  return s->prec == QCS_CUDA_C64 && s->sem == QCS_CUDA_PHYSICAL && k >= 5 && k <= 7 &&
         s->n >= k + 7 && s->n - k - 7 <= 40 && s->dev.cc_major == 10 && s->dev.cc_minor == 3;
}

template <int KA, int MODE>
static int launch_tc(qcs_cuda_state *s, const TcGeom &g, const uint4 *img, int renorm,
                     const double *diffuse_sum, ReduceSlot *sum_out) {
  using S = TcShape<KA>;
  static bool configured = false;
  if (!configured) {
    int rc = check_cuda(cudaFuncSetAttribute(k_block_tc<KA, MODE, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM),
                        "cudaFuncSetAttribute(tcgen05 block)");
    if (!rc)
      rc = check_cuda(cudaFuncSetAttribute(k_block_tc<KA, MODE, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM),
                      "cudaFuncSetAttribute(tcgen05 block, fused)");
    if (rc) return rc;
    configured = true;
  }
  const int grid = (int)(g.n_tiles < (i64)s->dev.num_sms ? g.n_tiles : s->dev.num_sms);
  prof_begin(s);
  if (diffuse_sum || sum_out)
    k_block_tc<KA, MODE, true><<<grid, kTcThreads, S::SMEM, s->stream>>>(
        (float2 *)s->vec, g, img, renorm, diffuse_sum, ldexp(1.0, -s->n), sum_out, s->d_err,
        wait_cycles());
  else
    k_block_tc<KA, MODE, false><<<grid, kTcThreads, S::SMEM, s->stream>>>(
        (float2 *)s->vec, g, img, renorm, nullptr, 0.0, nullptr, s->d_err, wait_cycles());
  return launched(s, KC_BLOCK_TC, 2.0 * s->size * 8.0, "apply_block (tcgen05)");
}

template <int MODE>
static int launch_tc7(qcs_cuda_state *s, const TcGeom &g, const uint4 *img, int renorm,
                      const double *diffuse_sum, ReduceSlot *sum_out) {
  static bool configured = false;
  if (!configured) {
    int rc = check_cuda(cudaFuncSetAttribute(k_block_tc7<MODE, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, Tc7::SMEM),
                        "cudaFuncSetAttribute(tcgen05 block, k = 7)");
    if (!rc)
      rc = check_cuda(cudaFuncSetAttribute(k_block_tc7<MODE, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, Tc7::SMEM),
                      "cudaFuncSetAttribute(tcgen05 block, k = 7, fused)");
    if (rc) return rc;
    configured = true;
  }
  const int grid = (int)(g.n_tiles < (i64)s->dev.num_sms ? g.n_tiles : s->dev.num_sms);
  prof_begin(s);
  if (diffuse_sum || sum_out)
    k_block_tc7<MODE, true><<<grid, Tc7::THREADS, Tc7::SMEM, s->stream>>>(
        (float2 *)s->vec, g, img, renorm, diffuse_sum, ldexp(1.0, -s->n), sum_out, s->d_err,
        wait_cycles());
  else
    k_block_tc7<MODE, false><<<grid, Tc7::THREADS, Tc7::SMEM, s->stream>>>(
        (float2 *)s->vec, g, img, renorm, nullptr, 0.0, nullptr, s->d_err, wait_cycles());
  return launched(s, KC_BLOCK_TC7, 2.0 * s->size * 8.0, "apply_block (tcgen05, k = 7)");
}

// Whether U is unitary (to FP64 rounding): unitary blocks get the
// per-column norm restore.  Checked as |U^H U v - v| <= 1e-9 |v| for two
// fixed pseudo-random vectors v, O(K^2) instead of the O(K^3) of forming
// U^H U: a non-unitary U has U^H U - I != 0, which a random v lies in the
// null space of with probability zero.
static bool is_unitary(const double *u, int K) {
  std::vector<double> v(2 * K), w(2 * K), x(2 * K);
  unsigned long long st = 0x9E3779B97F4A7C15ULL;
  for (int trial = 0; trial < 2; trial++) {
    double vn = 0.0;
    for (int i = 0; i < 2 * K; i++) {
      st = st * 6364136223846793005ULL + 1442695040888963407ULL;
      v[i] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
      vn += v[i] * v[i];
    }
    for (int r = 0; r < K; r++) {  // w = U v
      double re = 0.0, im = 0.0;
      for (int c = 0; c < K; c++) {
        const double ur = u[2 * (r * K + c)], ui = u[2 * (r * K + c) + 1];
        re += ur * v[2 * c] - ui * v[2 * c + 1];
        im += ur * v[2 * c + 1] + ui * v[2 * c];
      }
      w[2 * r] = re;
      w[2 * r + 1] = im;
    }
    for (int c = 0; c < K; c++) {  // x = U^H w
      double re = 0.0, im = 0.0;
      for (int r = 0; r < K; r++) {
        const double ur = u[2 * (r * K + c)], ui = -u[2 * (r * K + c) + 1];
        re += ur * w[2 * r] - ui * w[2 * r + 1];
        im += ur * w[2 * r + 1] + ui * w[2 * r];
      }
      x[2 * c] = re;
      x[2 * c + 1] = im;
    }
    double dn = 0.0;
    for (int i = 0; i < 2 * K; i++) dn += (x[i] - v[i]) * (x[i] - v[i]);
    if (!(dn <= 1e-18 * vn)) return false;
  }
  return true;
}

// A block made ready for the tensor cores: ascending qubits (the matrix
// relabelled to match), geometry, access mode, whether the norm is restored,
// and the image: split-BF16 B, then the matrix's row sums (float2) that a
// fused diffusion needs.
struct TcResident {
  int k = 0, mode = 0, renorm = 0;
  size_t image_bytes = 0;
  TcGeom g;
  std::vector<uint8_t> image;  // host copy
  uint8_t *dev = nullptr;      // device copy (resident blocks only)
};

static void tc_prepare(const qcs_cuda_state *s, int k, const int *qubits_in, const double *u_in,
                       bool known_unitary, TcResident &out) {
  const int KA = 1 << k;
  // Ascending qubits (block bit j = j-th smallest qubit), the matrix relabelled
  // to match: new index a' has bit j where the old index has bit order[j].
  int order[8], qubits[8];
  for (int j = 0; j < k; j++) order[j] = j;
  std::sort(order, order + k, [&](int x, int y) { return qubits_in[x] < qubits_in[y]; });
  bool sorted = true;
  for (int j = 0; j < k; j++) {
    qubits[j] = qubits_in[order[j]];
    sorted = sorted && order[j] == j;
  }
  std::vector<double> u_perm;
  const double *u = u_in;
  if (!sorted) {
    std::vector<int> old_of(KA);
    for (int a = 0; a < KA; a++) {
      int o = 0;
      for (int j = 0; j < k; j++)
        if ((a >> j) & 1) o |= 1 << order[j];
      old_of[a] = o;
    }
    u_perm.resize((size_t)2 * KA * KA);
    for (int a = 0; a < KA; a++)
      for (int b = 0; b < KA; b++) {
        const size_t src = 2 * ((size_t)old_of[a] * KA + old_of[b]);
        u_perm[2 * ((size_t)a * KA + b)] = u_in[src];
        u_perm[2 * ((size_t)a * KA + b) + 1] = u_in[src + 1];
      }
    u = u_perm.data();
  }
  // geometry
  TcGeom &g = out.g;
  memset(&g, 0, sizeof(g));
  std::vector<int> role(s->n, -1);  // >= 0 block bit, -2 column, -1 free
  for (int j = 0; j < k; j++) role[qubits[j]] = j;
  std::vector<int> colq;
  for (int q = 0; q < s->n && (int)colq.size() < 7; q++)
    if (role[q] == -1) {
      role[q] = -2;
      colq.push_back(q);
    }
  for (int q = 0; q < s->n; q++)
    if (role[q] == -1) g.freeq[g.nfree++] = (signed char)q;
  for (int k = 0; 4 * k < g.nfree; k++)
    for (int v = 0; v < 16; v++) {
      i64 o = 0;
      for (int b = 0; b < 4 && 4 * k + b < g.nfree; b++)
        if ((v >> b) & 1) o |= 1LL << g.freeq[4 * k + b];
      g.nib[k][v] = o;
    }
  g.n_tiles = 1LL << g.nfree;
  for (int m = 0; m < kTcM; m++) {
    i64 o = 0;
    for (int b = 0; b < 7; b++)
      if ((m >> b) & 1) o |= 1LL << colq[b];
    g.col_off[m] = o;
  }
  for (int a = 0; a < KA; a++) {
    i64 o = 0;
    for (int j = 0; j < k; j++)
      if ((a >> j) & 1) o |= 1LL << qubits[j];
    g.blk_off[a] = o;
  }
  {
    // the tile's qubits ascending; the lowest R of them are 0..R-1 (R >= 7),
    // so the tile is 2^(k+7-R) runs of 2^R adjacent amplitudes
    std::vector<int> tq;
    for (int q = 0; q < s->n; q++)
      if (role[q] != -1) tq.push_back(q);
    int R = 0;
    while (R < (int)tq.size() && tq[R] == R) R++;
    const int nt = (int)tq.size();
    // pieces: runs split down to at most 2^pf_piece amplitudes, at most 128
    const int nrun_bits = nt - R;
    int piece = R;
    while (piece > pf_piece_bits() && nrun_bits + (R - piece) < 7) piece--;
    g.nruns = 1 << (nrun_bits + (R - piece));
    g.run_bytes = (int)(8LL << piece);
    for (int j = 0; j < g.nruns; j++) {
      const int sub = j & ((1 << (R - piece)) - 1);  // piece within its run
      const int run = j >> (R - piece);
      i64 o = (i64)sub << piece;
      for (int b = R; b < nt; b++)
        if ((run >> (b - R)) & 1) o |= 1LL << tq[b];
      g.run_off[j] = o;
    }
    g.pf_ahead = pf_ahead(k);
  }
  bool low = true;  // the block is exactly qubits 0..k-1
  for (int j = 0; j < k; j++) low = low && qubits[j] == j;
  out.k = k;
  out.mode = low ? kLowMode : (qubits[0] == 0 ? kPairMode : kColMode);
  out.renorm = (known_unitary || is_unitary(u, KA)) ? 1 : 0;
  const size_t img = k == 7   ? Tc7::IMG_BYTES
                     : k == 6 ? TcShape<64>::IMG_BYTES
                              : TcShape<32>::IMG_BYTES;
  out.image_bytes = img + (size_t)KA * 8;
  out.image.assign(out.image_bytes, 0);
  if (k == 7) make_image7(u, out.image.data());
  else if (k == 6) make_image<64>(u, out.image.data());
  else make_image<32>(u, out.image.data());
  float *rows = reinterpret_cast<float *>(out.image.data() + img);
  for (int a = 0; a < KA; a++) {
    double re = 0.0, im = 0.0;
    for (int b = 0; b < KA; b++) {
      re += u[2 * ((size_t)a * KA + b)];
      im += u[2 * ((size_t)a * KA + b) + 1];
    }
    rows[2 * a] = (float)re;
    rows[2 * a + 1] = (float)im;
  }
}

// Launches a prepared block whose image is at `img` on the device.
static int tc_launch(qcs_cuda_state *s, const TcResident &b, const uint4 *img,
                     const BlockFuse *fuse) {
  const bool diffuse_in = fuse && fuse->diffuse_in;
  const bool sum_out = fuse && fuse->sum_out;
  int rc = QCS_CUDA_OK;
  if (diffuse_in) {
    rc = ensure_sum(s);  // m of the state the diffusion acts on
    if (rc) return rc;
  }
  const double *dsum = diffuse_in ? s->d_result + 4 : nullptr;
  ReduceSlot *sout = sum_out ? s->d_partials : nullptr;
  const TcGeom &g = b.g;
  if (b.k == 7)
    rc = b.mode == kLowMode    ? launch_tc7<kLowMode>(s, g, img, b.renorm, dsum, sout)
         : b.mode == kPairMode ? launch_tc7<kPairMode>(s, g, img, b.renorm, dsum, sout)
                               : launch_tc7<kColMode>(s, g, img, b.renorm, dsum, sout);
  else if (b.k == 6)
    rc = b.mode == kLowMode    ? launch_tc<64, kLowMode>(s, g, img, b.renorm, dsum, sout)
         : b.mode == kPairMode ? launch_tc<64, kPairMode>(s, g, img, b.renorm, dsum, sout)
                               : launch_tc<64, kColMode>(s, g, img, b.renorm, dsum, sout);
  else
    rc = b.mode == kLowMode    ? launch_tc<32, kLowMode>(s, g, img, b.renorm, dsum, sout)
         : b.mode == kPairMode ? launch_tc<32, kPairMode>(s, g, img, b.renorm, dsum, sout)
                               : launch_tc<32, kColMode>(s, g, img, b.renorm, dsum, sout);
  if (rc) return rc;
  invalidate_sum(s);
  if (sum_out) {
    const int grid = (int)(g.n_tiles < (i64)s->dev.num_sms ? g.n_tiles : s->dev.num_sms);
    rc = finalize_sum(s, grid * kTcEpiWarps);
  }
  return rc;
}

int apply_block_tc(qcs_cuda_state *s, int k, const int *qubits, const double *u,
                   bool known_unitary, const BlockFuse *fuse) {
  int rc = ring_init(s);
  if (rc) return rc;
  TcRing *r = s->tc;
  TcResident b;
  tc_prepare(s, k, qubits, u, known_unitary, b);
  // the image through the pinned ring
  const int slot = r->next;
  r->next = (r->next + 1) % kImgSlots;
  rc = check_cuda(cudaEventSynchronize(r->done[slot]), "block image slot");
  if (rc) return rc;
  uint8_t *h = r->host + slot * kImgSlotBytes;
  uint8_t *d = r->dev + slot * kImgSlotBytes;
  memcpy(h, b.image.data(), b.image_bytes);
  rc = copy_h2d(s, d, h, b.image_bytes, "block image upload");
  if (rc) return rc;
  rc = tc_launch(s, b, reinterpret_cast<const uint4 *>(d), fuse);
  if (rc) return rc;
  return check_cuda(cudaEventRecord(r->done[slot], s->stream), "block image event");
}

// Resident blocks: prepared once, image kept on the device, launched with no
// host-to-device traffic (kept plans).
int tc_make_resident(qcs_cuda_state *s, int k, const int *qubits, const double *u,
                     bool known_unitary, TcResident **out) {
  int rc = ring_init(s);
  if (rc) return rc;
  TcResident *b = new TcResident();
  tc_prepare(s, k, qubits, u, known_unitary, *b);
  rc = check_cuda(cudaMalloc((void **)&b->dev, b->image_bytes), "cudaMalloc(block image)");
  if (!rc) {  // through the pinned ring, so that the copy stays asynchronous
    TcRing *r = s->tc;
    const int slot = r->next;
    r->next = (r->next + 1) % kImgSlots;
    rc = check_cuda(cudaEventSynchronize(r->done[slot]), "block image slot");
    if (!rc) {
      memcpy(r->host + slot * kImgSlotBytes, b->image.data(), b->image_bytes);
      rc = copy_h2d(s, b->dev, r->host + slot * kImgSlotBytes, b->image_bytes,
                    "block image upload");
    }
    if (!rc) rc = check_cuda(cudaEventRecord(r->done[slot], s->stream), "block image event");
  }
  if (rc) {
    tc_free_resident(b);
    return rc;
  }
  b->image.clear();
  b->image.shrink_to_fit();
  *out = b;
  return QCS_CUDA_OK;
}

int tc_launch_resident(qcs_cuda_state *s, const TcResident *b, const BlockFuse *fuse) {
  return tc_launch(s, *b, reinterpret_cast<const uint4 *>(b->dev), fuse);
}

size_t tc_resident_bytes(const TcResident *b) { return b->image_bytes; }

void tc_free_resident(TcResident *b) {
  if (!b) return;
  if (b->dev) cudaFree(b->dev);
  delete b;
}

}  // namespace qcs

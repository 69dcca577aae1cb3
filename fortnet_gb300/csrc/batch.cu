// Batched mixed-precision form of the training and prediction passes (TBpnn_nTrain's epoch,
// lib_nn/bpnn.F90:147-390, with its gradient TBpnn_updateGradients 394-481 / sysTrain 610-704,
// and TBpnn_predictBatch 1001-1058), on Blackwell tensor cores.
//
// The dataset is cut into mini-batches of consecutive structures.  Inside a mini-batch the
// atoms of every species form 128-row tiles (zero rows pad each species' last tile).  The
// z-scored features of every tile are stored once, as BF16, already in the operand layout of
// tcgen05.mma (tc.cuh: core matrices, no swizzle), with a constant-1 column after the last
// feature that carries the first layer's bias through the GEMM.  One persistent kernel per
// stage walks a tile range with one CTA per SM:
//   * a bulk copy (cp.async.bulk, mbarrier completion) brings a tile's 128 x K0 features into
//     shared memory, and the species' packed BF16 weights when the species changes;
//   * layer GEMMs run as tcgen05.mma kind::f16 (BF16 x BF16, FP32 accumulators in TMEM, 128
//     lanes = 128 atoms); a thread owns one atom: tcgen05.ld brings its row of accumulators
//     into registers, tanh and the output layer (a 64-wide dot) run there, and the BF16
//     activations go back to shared memory as the next GEMM's operand;
//   * training adds the reverse pass: delta_2 in registers, delta_1 = (W_1 delta_2) * f'
//     as another GEMM, and the weight gradients X^T delta_1, a_1^T delta_2, a_2^T delta_3 as
//     GEMMs over the tile's rows (MN-major operands, the same buffers), accumulated in TMEM
//     over all tiles of the CTA and written once per CTA and species (FP32).
// The per-CTA gradient partials are summed in FP64 in a fixed order; the update is the
// reference's steepest descent (steepdesc.F90:126-204) on the FP64 master parameters,
// applied per mini-batch.  A whole epoch (every mini-batch: forward, loss, reverse pass,
// reduction, update) is captured once as a CUDA graph and replayed.  Launch shapes (CTAs per
// stage) are chosen by timing candidates on first use and kept per network shape.
//
// Supported networks: two hidden tanh layers of equal padded width 16, 32 or 64 (at most 64
// units each), one linear output, at most 239 inputs.
#define FNETG_FILE_CODE 5  // site codes of the bounds-checked build
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "internal.cuh"
#include "tc.cuh"

namespace fnetg {

__global__ void struct_sum_kernel(const double *out, const int64_t *off, int S, int nout,
                                  double *gsum);
int launch_loss_range(fnetg_ctx *ctx, int s0, int count, int loss);
int launch_loss_reduce(fnetg_ctx *ctx);

namespace {

constexpr int kRows = 128;          // atoms per tile (MMA M, TMEM lanes)
constexpr int kMaxTcBlocks = 1024;  // CTAs of one tensor-core launch (gradient partial slots)
constexpr int kThreads = 128;       // one thread per atom of the tile
constexpr uint32_t kTmemCols = 512;
// TMEM column regions
constexpr uint32_t kColFwd = 0;     // layer pre-activations / reverse-pass GEMM (<= 64 columns)
constexpr uint32_t kColG0 = 128;    // first-layer weight gradient, two 128-input M tiles
constexpr uint32_t kColG1 = 256;    // second-layer weight gradient
constexpr uint32_t kColG2 = 384;    // output-layer weight gradient (16 columns)

__host__ __device__ inline int rup(int x, int m) { return (x + m - 1) / m * m; }

struct TcNet {
  int nf, H1, H2;                    // real widths
  int K0p, K1p, K2p, nmt0;           // padded GEMM K of the three layers, M tiles of X^T delta
  uint32_t x_bytes;                  // one tile of packed features
  // one species' weight block: W0 | W1 forward | w2, b3 | W1 reverse | W0 reverse; the
  // forward pass loads the first w_bytes0, training and the tangent pass w_bytes1, the
  // Jacobian all w_bytes
  uint32_t w_bytes, w_bytes0, w_bytes1;
  uint32_t off_w1f, off_w1b, off_w0b, off_w2;  // offsets inside the weight block
  // shared-memory plan (bytes) of the training kernel (and of the Jacobian kernel, whose
  // weights end at jm_total): features | activations of both layers (exactly their K columns:
  // the 128-wide MN-major reads of the weight-gradient products run on into the next buffer) |
  // adjoints | weights | second feature buffer (the next tile's features, loaded while the
  // current tile computes; prefetch = 0 where it does not fit)
  uint32_t sm_x, sm_a1, sm_a2, sm_d2, sm_d1, sm_d3, sm_w, sm_x1, sm_total, jm_total;
  int prefetch;
  // shared-memory plan of the forward kernel: features, first activations, the weights it
  // reads; small enough for two CTAs per SM
  uint32_t fm_x, fm_a1, fm_w, fm_total;
  // shared-memory plan of the tangent (force-loss) kernel: features and their tangents,
  // activations and tangents of both hidden layers (exactly their K columns: the 128-wide
  // MN-major reads of a layer run on into the next buffer), adjoints, output adjoints, weights
  uint32_t tm_x, tm_u, tm_a1, tm_t1, tm_a2, tm_t2, tm_zb, tm_zd, tm_d3a, tm_d3b, tm_w, tm_total;
  // reference layout of one species' parameters (network.F90:397-427)
  int64_t nparams, woff0, woff1, woff2, woff3, boff1, boff2, boff3;
};

template <int HP> TcNet make_net(fnetg_ctx *ctx) {
  TcNet n{};
  n.nf = ctx->dims[0];
  n.H1 = ctx->dims[1];
  n.H2 = ctx->dims[2];
  n.K0p = rup(n.nf + 1, 16);
  n.K1p = rup(n.H1 + 1, 16);
  n.K2p = rup(n.H2 + 1, 16);
  n.nmt0 = (n.K0p + kRows - 1) / kRows;
  n.x_bytes = (uint32_t)kRows * n.K0p * 2;
  const uint32_t w0 = (uint32_t)HP * n.K0p * 2, w1f = (uint32_t)HP * n.K1p * 2,
                 w1b = (uint32_t)HP * HP * 2, w0b = (uint32_t)n.K0p * HP * 2,
                 w2 = (uint32_t)(HP + 4) * 4;
  n.off_w1f = w0;
  n.off_w2 = w0 + w1f;
  n.off_w1b = n.off_w2 + w2;
  n.off_w0b = n.off_w1b + w1b;
  n.w_bytes0 = n.off_w1b;  // multiples of 16: (HP + 4) * 4 and every image are
  n.w_bytes1 = n.off_w0b;
  n.w_bytes = n.off_w0b + w0b;
  // stored columns of a hidden layer's activations: the GEMM's K extent, and at least the HP
  // columns the epilogues write (K1p < HP when H1 < H2)
  const uint32_t k1s = (uint32_t)std::max(n.K1p, HP), k2s = (uint32_t)std::max(n.K2p, HP);
  uint32_t o = 0;
  n.sm_x = o;
  o += n.x_bytes;
  n.sm_a1 = o;
  o += kRows * k1s * 2;
  n.sm_a2 = o;
  o += kRows * k2s * 2;
  n.sm_d2 = o;
  o += kRows * HP * 2;
  n.sm_d1 = o;
  o += kRows * HP * 2;
  n.sm_d3 = o;
  o += kRows * 16 * 2;
  n.sm_w = o;
  n.sm_x1 = o + n.w_bytes1;
  n.jm_total = o + n.w_bytes;
  {
    // The MN-major operand reads run past a buffer's own columns: 128 columns of a_1 and a_2
    // (the M tile of a^T delta), nmt0 x 128 columns of a feature buffer (the M tiles of
    // X^T delta_1).  Every such read stays inside the allocation: the first feature buffer and
    // the activations are followed by other buffers; the second feature buffer closes the plan,
    // so the plan is extended by its over-read.
    const uint32_t mt_bytes = (uint32_t)n.nmt0 * kRows * kRows * 2;
    const uint32_t reach = std::max({n.sm_a1 + kRows * kRows * 2, n.sm_a2 + kRows * kRows * 2,
                                     n.sm_x + mt_bytes});
    const uint32_t with_x1 = std::max({n.sm_x1 + n.x_bytes, n.sm_x1 + mt_bytes, reach});
    n.prefetch = with_x1 <= 227u * 1024u - 1024u ? 1 : 0;
    n.sm_total = n.prefetch ? with_x1 : std::max(n.sm_x1, reach);
  }
  o = 0;
  n.fm_x = o;
  o += n.x_bytes;
  n.fm_a1 = o;  // only the K-major reads of the second layer
  o += kRows * k1s * 2;
  n.fm_w = o;
  o += n.w_bytes0;
  n.fm_total = o;
  o = 0;
  n.tm_x = o;
  o += n.x_bytes;
  n.tm_u = o;
  o += n.x_bytes;
  n.tm_a1 = o;
  o += kRows * k1s * 2;
  n.tm_t1 = o;
  o += kRows * k1s * 2;
  n.tm_a2 = o;
  o += kRows * k2s * 2;
  n.tm_t2 = o;
  o += kRows * k2s * 2;
  n.tm_zb = o;
  o += kRows * HP * 2;
  n.tm_zd = o;
  o += kRows * HP * 2;
  n.tm_d3a = o;
  o += kRows * 16 * 2;
  n.tm_d3b = o;
  o += kRows * 16 * 2;
  n.tm_w = o;
  o += n.w_bytes1;
  {
    // the transposed-operand reads (128 columns of an activation or tangent buffer, nmt0 x 128
    // of a feature or feature-tangent buffer) stay inside the allocation
    const uint32_t mt_bytes = (uint32_t)n.nmt0 * kRows * kRows * 2, m1 = kRows * kRows * 2;
    n.tm_total = std::max({o, n.tm_x + mt_bytes, n.tm_u + mt_bytes, n.tm_a1 + m1, n.tm_t1 + m1,
                           n.tm_a2 + m1, n.tm_t2 + m1});
  }
  n.nparams = ctx->nparams;
  n.woff0 = ctx->woff[0];
  n.woff1 = ctx->woff[1];
  n.woff2 = ctx->woff[2];
  n.woff3 = ctx->woff[3];
  n.boff1 = ctx->boff[1];
  n.boff2 = ctx->boff[2];
  n.boff3 = ctx->boff[3];
  return n;
}

struct TcArgs {
  TcNet net;
  const unsigned char *x;     // packed feature tiles
  const unsigned char *w;     // packed weights [nsp][w_bytes]
  const int32_t *tile_sp;     // species of every tile
  const int32_t *tile_atoms;  // [ntiles * 128] atom of every row, -1 = padding
  int64_t t0, t1;             // tile range of the launch
  double *out;                // [N] atomic outputs (forward)
  const double *delta;        // [N] scaled loss gradients of the outputs (training)
  float *gpart;               // [gridDim.x][nsp][nparams] gradient partials (training)
  int32_t *gflag;             // [gridDim.x][nsp] partial written
  int nsp;
  int *err;                   // set to 1 when a bounded wait gave up
  // Jacobian kernel: d out / d x of every atom, scaled by the inverse z-score deviations of
  // the ACSF columns, [N][nf] atom order (the force kernel's input)
  float *jac;
  const float *zinv;          // [ng] inverse deviations, 0 = not standardised
  int ng;
  // tangent kernel: packed BF16 tangents of the inputs, same tiles and layout as x
  const unsigned char *u;
  int64_t natoms;             // atoms of the context (bounds-checked build)
};

// A tile row's atom; in the bounds-checked build an index outside the context's atoms is
// recorded and the row treated as padding.
__device__ __forceinline__ int tile_atom(const int32_t *tile_atoms, int64_t k, int64_t natoms) {
  const int v = tile_atoms[k];
  return (v < 0 || FNETG_GUARD(v < natoms)) ? v : -1;
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&p);
}
__device__ __forceinline__ void st8(unsigned char *base, uint32_t off, const float *v) {
  *reinterpret_cast<uint4 *>(base + off) =
      make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

// every thread polls; the outcome is made uniform across the CTA
__device__ __forceinline__ bool wait_all(uint64_t *mb, uint32_t parity) {
  const bool ok = tc::mbar_wait(mb, parity);
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

// Row r's activations of one hidden layer to shared memory as BF16 (core layout, 128 rows):
// columns [0, HP) from v, then the constant-1 column at index H and zeros up to Kp.
template <int HP>
__device__ __forceinline__ void store_act(unsigned char *buf, int r, float (&v)[HP], int H,
                                          int Kp) {
#pragma unroll
  for (int c = 0; c < HP; c++)
    if (c == H) v[c] = 1.f;  // unrolled compare: the array stays in registers
#pragma unroll
  for (int c = 0; c < HP; c += 8) st8(buf, tc::core_off(r, c, kRows), v + c);
  if (H >= HP) {
    float e[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(buf, tc::core_off(r, HP, kRows), e);
    float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c = HP + 8; c < Kp; c += 8) st8(buf, tc::core_off(r, c, kRows), z);
  }
}

// Row r's tangents of one hidden layer (BF16, core layout): columns [0, HP) from v (padded
// units carry zero tangents), zeros in the bias column and up to Kp.
template <int HP>
__device__ __forceinline__ void store_tan(unsigned char *buf, int r, const float (&v)[HP], int H,
                                          int Kp) {
#pragma unroll
  for (int c = 0; c < HP; c += 8) st8(buf, tc::core_off(r, c, kRows), v + c);
  if (H >= HP) {
    float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c = HP; c < Kp; c += 8) st8(buf, tc::core_off(r, c, kRows), z);
  }
}

// eight BF16 values of a core row back to floats
__device__ __forceinline__ void ld8(const unsigned char *base, uint32_t off, float *v) {
  const uint4 q = *reinterpret_cast<const uint4 *>(base + off);
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    __nv_bfloat162 p;
    *reinterpret_cast<uint32_t *>(&p) = w[k];
    v[2 * k] = __low2float(p);
    v[2 * k + 1] = __high2float(p);
  }
}

// nk MMAs of K = 16 accumulating into d: operands advance by a_step / b_step bytes per step
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a0, uint32_t a_lbo, uint32_t a_sbo,
                                          uint32_t a_step, uint32_t b0, uint32_t b_lbo,
                                          uint32_t b_sbo, uint32_t b_step, int nk, uint32_t idesc,
                                          bool acc) {
  for (int ks = 0; ks < nk; ks++)
    tc::mma_bf16(d, tc::smem_desc(a0 + ks * a_step, a_lbo, a_sbo),
                 tc::smem_desc(b0 + ks * b_step, b_lbo, b_sbo), idesc, (acc || ks > 0) ? 1u : 0u);
}

// One gradient partial: stored, or added to what the same CTA stored for the species before
// (a launch over several mini-batches meets a species once per mini-batch).  A template flag,
// so that a plain flush issues no load of the old partial.
template <bool ADD> __device__ __forceinline__ void put_grad(float *p, float v) {
  if (ADD) *p += v;
  else *p = v;
}

// The TMEM gradient accumulators (G0 in M tiles of 128 inputs, G1, G2) -> one partial slot in
// the reference parameter order (all threads; thread tid holds lane tid of every region).
template <int HP, bool ADD>
__device__ void flush_grads(const TcNet &n, float *gp, uint32_t tm, uint32_t lane_off, int tid) {
  for (int mt = 0; mt < n.nmt0; mt++) {
    const int k = mt * kRows + tid;  // input feature (k == nf: the bias column)
#pragma unroll
    for (int c0 = 0; c0 < HP; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tm + lane_off + kColG0 + mt * HP + c0, v);
      tc::tmem_wait_ld();
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int j = c0 + q;
        if (j < n.H1 && k < n.nf) put_grad<ADD>(gp + n.woff0 + k + (int64_t)n.nf * j, v[q]);
        else if (j < n.H1 && k == n.nf) put_grad<ADD>(gp + n.boff1 + j, v[q]);
      }
    }
  }
#pragma unroll
  for (int c0 = 0; c0 < HP; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tm + lane_off + kColG1 + c0, v);
    tc::tmem_wait_ld();
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const int i = c0 + q;
      if (i < n.H2 && tid < n.H1) put_grad<ADD>(gp + n.woff1 + tid + (int64_t)n.H1 * i, v[q]);
      else if (i < n.H2 && tid == n.H1) put_grad<ADD>(gp + n.boff2 + i, v[q]);
    }
  }
  float v[16];
  tc::tmem_ld16(tm + lane_off + kColG2, v);
  tc::tmem_wait_ld();
  if (tid < n.H2) put_grad<ADD>(gp + n.woff2 + tid, v[0]);
  else if (tid == n.H2) put_grad<ADD>(gp + n.boff3, v[0]);
}

// Row r's activations of one hidden layer, the CH columns [c0, c0 + CH) of one half of the
// row (BF16, core layout): the constant-1 column at index H when it falls in this half; the
// half holding column HP also writes the constant column and the zero padding up to Kp when
// H == HP.
template <int HP, int CH>
__device__ __forceinline__ void store_act_half(unsigned char *buf, int r, float (&v)[CH], int c0,
                                               int H, int Kp) {
#pragma unroll
  for (int c = 0; c < CH; c++)
    if (c0 + c == H) v[c] = 1.f;  // unrolled compare: the array stays in registers
#pragma unroll
  for (int c = 0; c < CH; c += 8) st8(buf, tc::core_off(r, c0 + c, kRows), v + c);
  if (H >= HP && c0 + CH == HP) {
    float e[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(buf, tc::core_off(r, HP, kRows), e);
    float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c = HP + 8; c < Kp; c += 8) st8(buf, tc::core_off(r, c, kRows), z);
  }
}

// Gradient accumulators -> one CTA's partial slot (reference parameter order); thread (row,
// half) writes the columns of its half.
template <int HP, bool ADD>
__device__ void flush_grads_half(const TcNet &n, float *gp, uint32_t tm, uint32_t lane_off,
                                 int row, int half) {
  constexpr int CH = HP / 2;
  const int c0 = half * CH;
  for (int mt = 0; mt < n.nmt0; mt++) {
    const int k = mt * kRows + row;  // input feature (k == nf: the bias column)
    float v[CH];
    tc::tmem_ld_cols<CH>(tm + lane_off + kColG0 + mt * HP + c0, v);
#pragma unroll
    for (int q = 0; q < CH; q++) {
      const int j = c0 + q;
      if (j < n.H1 && k < n.nf) put_grad<ADD>(gp + n.woff0 + k + (int64_t)n.nf * j, v[q]);
      else if (j < n.H1 && k == n.nf) put_grad<ADD>(gp + n.boff1 + j, v[q]);
    }
  }
  {
    float v[CH];
    tc::tmem_ld_cols<CH>(tm + lane_off + kColG1 + c0, v);
#pragma unroll
    for (int q = 0; q < CH; q++) {
      const int i = c0 + q;
      if (i < n.H2 && row < n.H1) put_grad<ADD>(gp + n.woff1 + row + (int64_t)n.H1 * i, v[q]);
      else if (i < n.H2 && row == n.H1) put_grad<ADD>(gp + n.boff2 + i, v[q]);
    }
  }
  if (half == 0) {  // whole warps: the TMEM load is warp-collective
    float v[8];
    tc::tmem_ld_cols<8>(tm + lane_off + kColG2, v);
    if (row < n.H2) put_grad<ADD>(gp + n.woff2 + row, v[0]);
    else if (row == n.H2) put_grad<ADD>(gp + n.boff3, v[0]);
  }
}

// MODE 0: forward (atomic outputs).  MODE 1: forward + reverse pass + weight gradients.
// Two threads per atom row: warps w and w + 4 read the same TMEM lane quarter and split the
// hidden units of every epilogue (CH = HP / 2 columns each), so each scheduler runs two warps.
constexpr int kMlpThreads = 2 * kRows;
template <int HP, int MODE>
__global__ void __launch_bounds__(kMlpThreads, MODE == 0 ? 2 : 1) tc_mlp_kernel(TcArgs a) {
  constexpr int CH = HP / 2;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mb_load, mb_mma, mb_x[2];
  __shared__ uint32_t tmem_base;
  __shared__ float ypart[kRows];
  const TcNet &n = a.net;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (kRows - 1), half = tid >> 7, c0 = half * CH;
  // the forward pass uses its own compact plan (two CTAs per SM) and 64 TMEM columns
  constexpr uint32_t kCols = MODE == 0 ? 64u : kTmemCols;
  const uint32_t wload = MODE == 0 ? n.w_bytes0 : n.w_bytes1;
  unsigned char *X = sm + (MODE == 0 ? n.fm_x : n.sm_x), *A1 = sm + (MODE == 0 ? n.fm_a1 : n.sm_a1),
                *A2 = sm + n.sm_a2, *D2 = sm + n.sm_d2, *D1 = sm + n.sm_d1, *D3 = sm + n.sm_d3,
                *W = sm + (MODE == 0 ? n.fm_w : n.sm_w);
  // training: the next tile's features are requested into the other buffer while the current
  // tile computes (mb_x[b] counts buffer b's copy; mb_load the weights)
  const bool pf = MODE == 1 && n.prefetch;
  unsigned char *const Xb0 = X, *const Xb1 = sm + n.sm_x1;
  const float *w2 = reinterpret_cast<const float *>(W + n.off_w2);
  if (tid == 0) {
    tc::mbar_init(&mb_load, 1);
    tc::mbar_init(&mb_mma, 1);
    tc::mbar_init(&mb_x[0], 1);
    tc::mbar_init(&mb_x[1], 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  const uint32_t sA1 = tc::smem_u32(A1), sA2 = tc::smem_u32(A2),
                 sD2 = tc::smem_u32(D2), sD1 = tc::smem_u32(D1), sD3 = tc::smem_u32(D3),
                 sW = tc::smem_u32(W);
  // K-major operands (tc.cuh): lbo = 16 * rows, sbo = 128; MN-major: lbo = 128, sbo = 16 * rows
  const uint32_t id_h = tc::idesc_bf16(kRows, HP, 0, 0);
  const uint32_t id_g = tc::idesc_bf16(kRows, HP, 1, 1);
  const uint32_t id_g2 = tc::idesc_bf16(kRows, 16, 1, 1);
  uint32_t ph_load = 0, ph_mma = 0, ph_x0 = 0, ph_x1 = 0;
  bool pend_x0 = false, pend_x1 = false, pend_w = false;  // copies requested, not yet waited for
  const int64_t nt = a.t1 - a.t0;
  const int64_t my0 = a.t0 + nt * blockIdx.x / gridDim.x;
  const int64_t my1 = a.t0 + nt * (blockIdx.x + 1) / gridDim.x;
  int cur_sp = -1;
  bool gacc = false;  // the TMEM gradient accumulators hold data of cur_sp
  uint64_t touched = 0;
  bool failed = false;
  int buf = 0;
  // With the feature prefetch, a tile's input-layer weight gradient G0 += X^T delta_1 is issued
  // after the next tile's first-layer MMAs (so it runs under that tile's epilogue instead of
  // ahead of it); until then it is pending with its feature buffer and accumulate flag.
  bool g0_pend = false, g0_acc = false;
  uint32_t g0_x = 0;

  // G0 += X^T delta_1 over the input features in M tiles of 128 (issuing thread only)
  auto issue_g0 = [&](uint32_t sx, bool acc) {
    for (int mt = 0; mt < n.nmt0; mt++)
      for (int ks = 0; ks < kRows / 16; ks++)
        tc::mma_bf16(tm + kColG0 + mt * HP,
                     tc::smem_desc(sx + mt * 16 * 16 * kRows + ks * 256, 128, 16 * kRows),
                     tc::smem_desc(sD1 + ks * 256, 128, 16 * kRows), id_g, acc || ks > 0);
  };
  // every MMA issued so far (a pending G0 first) has completed: the TMEM accumulators are final
  auto settle = [&]() -> bool {
    if (tid == 0) {
      tc::fence_after_sync();
      if (g0_pend) issue_g0(g0_x, g0_acc);
      tc::mma_commit(&mb_mma);
    }
    g0_pend = false;
    if (!wait_all(&mb_mma, ph_mma)) return false;
    ph_mma ^= 1;
    tc::fence_after_sync();
    return true;
  };
  // gradient accumulators of cur_sp -> this CTA's partial slot (reference parameter order)
  auto flush = [&]() {
    float *gp = a.gpart + ((int64_t)blockIdx.x * a.nsp + cur_sp) * n.nparams;
    if ((touched >> cur_sp) & 1) flush_grads_half<HP, true>(n, gp, tm, lane_off, row, half);
    else flush_grads_half<HP, false>(n, gp, tm, lane_off, row, half);
    touched |= 1ull << cur_sp;
  };
  // after a wait gave up: the copies still in flight, each once more with a limit
  auto drain = [&]() {
    if (pend_w) tc::mbar_wait(&mb_load, ph_load);
    if (pend_x0) tc::mbar_wait(&mb_x[0], ph_x0);
    if (pend_x1) tc::mbar_wait(&mb_x[1], ph_x1);
  };

  if (pf && my0 < my1) {
    if (tid == 0) {
      tc::mbar_expect_tx(&mb_x[0], n.x_bytes);
      tc::bulk_g2s(Xb0, a.x + my0 * (int64_t)n.x_bytes, n.x_bytes, &mb_x[0]);
    }
    pend_x0 = true;
  }
  // the tile's species, its rows' atoms and loss gradients are requested one tile ahead (the
  // gradient once the atom has arrived, half a tile later), off the tile's critical path
  int sp_next = my0 < my1 ? a.tile_sp[my0] : 0;
  int atom_next = my0 < my1 ? tile_atom(a.tile_atoms, my0 * kRows + row, a.natoms) : -1;
  float d3_next = (MODE == 1 && atom_next >= 0) ? (float)a.delta[atom_next] : 0.f;
  for (int64_t t = my0; t < my1; t++) {
    const int sp = sp_next;
    const int atom = atom_next;
    const float delta3 = d3_next;
    if (t + 1 < my1) {
      sp_next = a.tile_sp[t + 1];
      atom_next = tile_atom(a.tile_atoms, (t + 1) * kRows + row, a.natoms);
    }
    const bool new_sp = sp != cur_sp;
    if (MODE == 1 && new_sp && gacc) {
      if (!settle()) {
        drain();
        failed = true;
        break;
      }
      flush();
      gacc = false;
    }
    tc::fence_before_sync();
    __syncthreads();
    const bool more = pf && t + 1 < my1;
    if (tid == 0) {
      if (pf) {
        // the weights' last readers (the previous species' layer and reverse MMAs) completed
        // before the flush; the next tile's features are requested after this tile's second
        // layer (below), once the other buffer's last reader has completed
        if (new_sp) {
          tc::mbar_expect_tx(&mb_load, wload);
          tc::bulk_g2s(W, a.w + (int64_t)sp * n.w_bytes, wload, &mb_load);
        }
      } else {
        tc::mbar_expect_tx(&mb_load, n.x_bytes + (new_sp ? wload : 0u));
        tc::bulk_g2s(X, a.x + t * (int64_t)n.x_bytes, n.x_bytes, &mb_load);
        if (new_sp) tc::bulk_g2s(W, a.w + (int64_t)sp * n.w_bytes, wload, &mb_load);
      }
    }
    if (pf) {
      pend_w = new_sp;
    } else {
      pend_w = true;
    }
    cur_sp = sp;
    if (pf) {
      if (!wait_all(&mb_x[buf], buf ? ph_x1 : ph_x0)) {
        drain();
        failed = true;
        break;
      }
      (buf ? ph_x1 : ph_x0) ^= 1;
      (buf ? pend_x1 : pend_x0) = false;
    }
    if (pend_w) {
      if (!wait_all(&mb_load, ph_load)) {
        drain();
        failed = true;
        break;
      }
      ph_load ^= 1;
      pend_w = false;
    }
    const uint32_t sX = tc::smem_u32(pf && buf ? Xb1 : Xb0);
    // ---- layer 1: Z1 = X W0 (+ bias through the constant column)
    if (tid == 0) {
      tc::fence_after_sync();
      for (int ks = 0; ks < n.K0p / 16; ks++)
        tc::mma_bf16(tm + kColFwd, tc::smem_desc(sX + ks * 2 * 16 * kRows, 16 * kRows, 128),
                     tc::smem_desc(sW + ks * 2 * 16 * HP, 16 * HP, 128), id_h, ks > 0);
      tc::mma_commit(&mb_mma);
      // the previous tile's G0 after this commit: it runs under this tile's epilogue and is
      // covered by the second layer's commit
      if (MODE == 1 && g0_pend) issue_g0(g0_x, g0_acc);
    }
    g0_pend = false;
    if (!wait_all(&mb_mma, ph_mma)) { drain(); failed = true; break; }
    ph_mma ^= 1;
    tc::fence_after_sync();
    if (MODE == 1 && t + 1 < my1) d3_next = atom_next >= 0 ? (float)a.delta[atom_next] : 0.f;
    float f1[CH];
    {
      float v[CH];
      tc::tmem_ld_cols<CH>(tm + lane_off + kColFwd + c0, v);
#pragma unroll
      for (int q = 0; q < CH; q++) {
        const float th = tanh_fast(v[q]);
        v[q] = th;
        f1[q] = 1.f - th * th;
      }
      store_act_half<HP, CH>(A1, row, v, c0, n.H1, n.K1p);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // ---- layer 2: Z2 = A1 W1 (+ bias)
    if (tid == 0) {
      tc::fence_after_sync();
      for (int ks = 0; ks < n.K1p / 16; ks++)
        tc::mma_bf16(tm + kColFwd, tc::smem_desc(sA1 + ks * 2 * 16 * kRows, 16 * kRows, 128),
                     tc::smem_desc(sW + n.off_w1f + ks * 2 * 16 * HP, 16 * HP, 128), id_h,
                     ks > 0);
      tc::mma_commit(&mb_mma);
    }
    if (!wait_all(&mb_mma, ph_mma)) { drain(); failed = true; break; }
    ph_mma ^= 1;
    tc::fence_after_sync();
    if (more) {
      // the other feature buffer's last reader, the previous tile's G0, has completed (this
      // commit covers it): the next tile's features go there
      if (tid == 0) {
        tc::mbar_expect_tx(&mb_x[buf ^ 1], n.x_bytes);
        tc::bulk_g2s(buf ? Xb0 : Xb1, a.x + (t + 1) * (int64_t)n.x_bytes, n.x_bytes,
                     &mb_x[buf ^ 1]);
      }
      (buf ? pend_x0 : pend_x1) = true;
    }
    {
      float y = 0.f;  // this half's share of w2 . a2
      float av[CH], dv[CH];
      tc::tmem_ld_cols<CH>(tm + lane_off + kColFwd + c0, av);
#pragma unroll
      for (int q = 0; q < CH; q++) {
        const float th = tanh_fast(av[q]);
        const float wq = w2[c0 + q];
        y = fmaf(th, wq, y);
        av[q] = th;
        dv[q] = delta3 * wq * (1.f - th * th);
      }
      if (MODE == 0) {
        // output = b3 + both halves' shares, added in a fixed order
        if (half == 1) ypart[row] = y;
        __syncthreads();
        if (half == 0 && atom >= 0) a.out[atom] = (double)(w2[HP] + (y + ypart[row]));
      } else {
        store_act_half<HP, CH>(A2, row, av, c0, n.H2, n.K2p);
#pragma unroll
        for (int c = 0; c < CH; c += 8) st8(D2, tc::core_off(row, c0 + c, kRows), dv + c);
        if (half == 0) {
          float d3[8] = {delta3, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          float z8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
          st8(D3, tc::core_off(row, 0, kRows), d3);
          st8(D3, tc::core_off(row, 8, kRows), z8);
        }
      }
    }
    if (MODE == 0) continue;
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // ---- reverse pass: P = delta_2 W1^T; G1 += A1^T delta_2; G2 += A2^T delta_3.  The
    // commit covers P only: the weight-gradient products run under the epilogue, and the next
    // commit (the next tile's first layer, or a flush) covers them before their operands change
    if (tid == 0) {
      tc::fence_after_sync();
      for (int ks = 0; ks < HP / 16; ks++)
        tc::mma_bf16(tm + kColFwd, tc::smem_desc(sD2 + ks * 2 * 16 * kRows, 16 * kRows, 128),
                     tc::smem_desc(sW + n.off_w1b + ks * 2 * 16 * HP, 16 * HP, 128), id_h,
                     ks > 0);
      tc::mma_commit(&mb_mma);
      for (int ks = 0; ks < kRows / 16; ks++) {
        tc::mma_bf16(tm + kColG1, tc::smem_desc(sA1 + ks * 256, 128, 16 * kRows),
                     tc::smem_desc(sD2 + ks * 256, 128, 16 * kRows), id_g, gacc || ks > 0);
        tc::mma_bf16(tm + kColG2, tc::smem_desc(sA2 + ks * 256, 128, 16 * kRows),
                     tc::smem_desc(sD3 + ks * 256, 128, 16 * kRows), id_g2, gacc || ks > 0);
      }
    }
    if (!wait_all(&mb_mma, ph_mma)) { drain(); failed = true; break; }
    ph_mma ^= 1;
    tc::fence_after_sync();
    {
      float dv[CH];
      tc::tmem_ld_cols<CH>(tm + lane_off + kColFwd + c0, dv);
#pragma unroll
      for (int q = 0; q < CH; q++) dv[q] *= f1[q];
#pragma unroll
      for (int c = 0; c < CH; c += 8) st8(D1, tc::core_off(row, c0 + c, kRows), dv + c);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    // ---- G0 += X^T delta_1 (input features in M tiles of 128): with the prefetch it waits
    // for the next tile's first layer (or a flush); without it, the next tile's features
    // overwrite this buffer, so it runs now
    if (pf) {
      g0_pend = true;
      g0_acc = gacc;
      g0_x = sX;
    } else {
      if (tid == 0) {
        tc::fence_after_sync();
        issue_g0(sX, gacc);
        tc::mma_commit(&mb_mma);
      }
      if (!wait_all(&mb_mma, ph_mma)) { drain(); failed = true; break; }
      ph_mma ^= 1;
      tc::fence_after_sync();
    }
    gacc = true;
    if (pf) buf ^= 1;
  }
  if (MODE == 1 && !failed) {
    if (gacc) {
      if (settle()) flush();
      else failed = true;
    }
    if (!failed && tid < a.nsp)
      a.gflag[(int64_t)blockIdx.x * a.nsp + tid] = (int)((touched >> tid) & 1);
  }
  if (failed && tid == 0) atomicExch(a.err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, kCols);
}

// CTA-uniform bounded wait that gives up the tile loop (a macro: it breaks the caller's loop)
#define TC_WAIT(mb, ph)            \
  if (!wait_all(&(mb), (ph))) {    \
    failed = true;                 \
    break;                         \
  }                                \
  (ph) ^= 1;                       \
  tc::fence_after_sync()

// make generic-proxy shared-memory writes visible to the MMAs, then hand over to the issuer
__device__ __forceinline__ void publish_smem() {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
}

// d out / d x of every atom (the input Jacobian of TNetwork_fdevi, network.F90:183-244, in
// reverse mode): forward, delta_2 = w2 * f'(z2) with seed 1, delta_1 = (W1 delta_2) * f'(z1),
// J = W0 delta_1 as a fourth GEMM (N = the padded inputs), each column scaled by its inverse
// z-score deviation for the force contraction.  The atomic outputs are written as well.
template <int HP>
__global__ void __launch_bounds__(kThreads, 1) tc_jac_kernel(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mb_load, mb_mma;
  __shared__ uint32_t tmem_base;
  const TcNet &n = a.net;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *X = sm + n.sm_x, *A1 = sm + n.sm_a1, *D2 = sm + n.sm_d2, *D1 = sm + n.sm_d1,
                *W = sm + n.sm_w;
  const float *w2 = reinterpret_cast<const float *>(W + n.off_w2);
  if (tid == 0) {
    tc::mbar_init(&mb_load, 1);
    tc::mbar_init(&mb_mma, 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base, lane_off = (uint32_t)(warp * 32) << 16;
  const uint32_t sX = tc::smem_u32(X), sA1 = tc::smem_u32(A1), sD2 = tc::smem_u32(D2),
                 sD1 = tc::smem_u32(D1), sW = tc::smem_u32(W);
  const uint32_t id_h = tc::idesc_bf16(kRows, HP, 0, 0), id_j = tc::idesc_bf16(kRows, n.K0p, 0, 0);
  constexpr uint32_t kColJ = 256;
  uint32_t ph_load = 0, ph_mma = 0;
  const int64_t nt = a.t1 - a.t0;
  const int64_t my0 = a.t0 + nt * blockIdx.x / gridDim.x;
  const int64_t my1 = a.t0 + nt * (blockIdx.x + 1) / gridDim.x;
  int cur_sp = -1;
  bool failed = false;
  for (int64_t t = my0; t < my1; t++) {
    const int sp = a.tile_sp[t];
    const bool new_sp = sp != cur_sp;
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::mbar_expect_tx(&mb_load, n.x_bytes + (new_sp ? n.w_bytes : 0u));
      tc::bulk_g2s(X, a.x + t * (int64_t)n.x_bytes, n.x_bytes, &mb_load);
      if (new_sp) tc::bulk_g2s(W, a.w + (int64_t)sp * n.w_bytes, n.w_bytes, &mb_load);
    }
    cur_sp = sp;
    const int row = tid;
    const int atom = tile_atom(a.tile_atoms, t * kRows + row, a.natoms);
    if (!wait_all(&mb_load, ph_load)) {
      tc::mbar_wait(&mb_load, ph_load);
      failed = true;
      break;
    }
    ph_load ^= 1;
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sX, 16 * kRows, 128, 32 * kRows, sW, 16 * HP, 128, 32 * HP, n.K0p / 16, id_h,
                false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    float f1[HP];
    {
      float v[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float z[16];
        tc::tmem_ld16(tm + lane_off + c0, z);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const float th = tanh_fast(z[q]);
          v[c0 + q] = th;
          f1[c0 + q] = 1.f - th * th;
        }
      }
      store_act<HP>(A1, row, v, n.H1, n.K1p);
    }
    publish_smem();
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sA1, 16 * kRows, 128, 32 * kRows, sW + n.off_w1f, 16 * HP, 128, 32 * HP,
                n.K1p / 16, id_h, false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    {
      float y = w2[HP], dv[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float z[16];
        tc::tmem_ld16(tm + lane_off + c0, z);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const float th = tanh_fast(z[q]);
          y = fmaf(th, w2[c0 + q], y);
          dv[c0 + q] = w2[c0 + q] * (1.f - th * th);
        }
      }
      if (atom >= 0) a.out[atom] = (double)y;
#pragma unroll
      for (int c = 0; c < HP; c += 8) st8(D2, tc::core_off(row, c, kRows), dv + c);
    }
    publish_smem();
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sD2, 16 * kRows, 128, 32 * kRows, sW + n.off_w1b, 16 * HP, 128, 32 * HP,
                HP / 16, id_h, false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    {
      float dv[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float z[16];
        tc::tmem_ld16(tm + lane_off + c0, z);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 16; q++) dv[c0 + q] = z[q] * f1[c0 + q];
      }
#pragma unroll
      for (int c = 0; c < HP; c += 8) st8(D1, tc::core_off(row, c, kRows), dv + c);
    }
    publish_smem();
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm + kColJ, sD1, 16 * kRows, 128, 32 * kRows, sW + n.off_w0b, 16 * n.K0p, 128,
                32 * n.K0p, HP / 16, id_j, false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    for (int c0 = 0; c0 < n.K0p; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tm + lane_off + kColJ + c0, v);
      tc::tmem_wait_ld();
      if (atom >= 0) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int k = c0 + q;
          if (k < n.nf) {
            float s = 1.f;
            if (k < a.ng) {
              const float inv = a.zinv[k];
              s = inv == 0.f ? 1.f : inv;
            }
            a.jac[(int64_t)atom * n.nf + k] = v[q] * s;
          }
        }
      }
    }
  }
  if (failed && tid == 0) atomicExch(a.err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, kTmemCols);
}

// The reverse pass of the force-loss gradient (forceloss.cu states the mathematics) on tensor
// cores: per tile the values and tangents of both hidden layers (X W0 and U W0, A1 W1 and
// T1 W1), the adjoints of the pre-activations and of their tangents (output adjoints: the
// energy loss gradient and -1), and the weight gradients X^T zbar_1 + U^T zdotbar_1,
// A1^T zbar_2 + T1^T zdotbar_2, A2^T ybar + T2^T ydotbar accumulated in TMEM as in the
// training kernel.
template <int HP>
__global__ void __launch_bounds__(kThreads, 1) tc_tan_kernel(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mb_load, mb_mma;
  __shared__ uint32_t tmem_base;
  const TcNet &n = a.net;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *X = sm + n.tm_x, *U = sm + n.tm_u, *A1 = sm + n.tm_a1, *T1 = sm + n.tm_t1,
                *A2 = sm + n.tm_a2, *T2 = sm + n.tm_t2, *ZB = sm + n.tm_zb, *ZD = sm + n.tm_zd,
                *D3a = sm + n.tm_d3a, *D3b = sm + n.tm_d3b, *W = sm + n.tm_w;
  const float *w2 = reinterpret_cast<const float *>(W + n.off_w2);
  if (tid == 0) {
    tc::mbar_init(&mb_load, 1);
    tc::mbar_init(&mb_mma, 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_base, lane_off = (uint32_t)(warp * 32) << 16;
  const uint32_t sX = tc::smem_u32(X), sU = tc::smem_u32(U), sA1 = tc::smem_u32(A1),
                 sT1 = tc::smem_u32(T1), sA2 = tc::smem_u32(A2), sT2 = tc::smem_u32(T2),
                 sZB = tc::smem_u32(ZB), sZD = tc::smem_u32(ZD), sD3a = tc::smem_u32(D3a),
                 sD3b = tc::smem_u32(D3b), sW = tc::smem_u32(W);
  const uint32_t id_h = tc::idesc_bf16(kRows, HP, 0, 0);
  const uint32_t id_g = tc::idesc_bf16(kRows, HP, 1, 1);
  const uint32_t id_g2 = tc::idesc_bf16(kRows, 16, 1, 1);
  constexpr uint32_t kColTan = 64;  // tangents next to the values
  uint32_t ph_load = 0, ph_mma = 0;
  const int64_t nt = a.t1 - a.t0;
  const int64_t my0 = a.t0 + nt * blockIdx.x / gridDim.x;
  const int64_t my1 = a.t0 + nt * (blockIdx.x + 1) / gridDim.x;
  int cur_sp = -1;
  bool gacc = false, failed = false;
  uint64_t touched = 0;
  // gradient accumulators of species sp -> this CTA's partial slot (added to an earlier one)
  auto flush_tan = [&](int sp) {
    float *gp = a.gpart + ((int64_t)blockIdx.x * a.nsp + sp) * n.nparams;
    if ((touched >> sp) & 1) flush_grads<HP, true>(n, gp, tm, lane_off, tid);
    else flush_grads<HP, false>(n, gp, tm, lane_off, tid);
  };
  // K-major: lbo 16 R, sbo 128, step 32 R; MN-major over 128 rows: lbo 128, sbo 2048, step 256
  for (int64_t t = my0; t < my1; t++) {
    const int sp = a.tile_sp[t];
    const bool new_sp = sp != cur_sp;
    if (new_sp && gacc) {
      flush_tan(cur_sp);
      touched |= 1ull << cur_sp;
      gacc = false;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::mbar_expect_tx(&mb_load, 2 * n.x_bytes + (new_sp ? n.w_bytes1 : 0u));
      tc::bulk_g2s(X, a.x + t * (int64_t)n.x_bytes, n.x_bytes, &mb_load);
      tc::bulk_g2s(U, a.u + t * (int64_t)n.x_bytes, n.x_bytes, &mb_load);
      if (new_sp) tc::bulk_g2s(W, a.w + (int64_t)sp * n.w_bytes, n.w_bytes1, &mb_load);
    }
    cur_sp = sp;
    const int row = tid;
    const int atom = tile_atom(a.tile_atoms, t * kRows + row, a.natoms);
    const float ybar = atom >= 0 ? (float)a.delta[atom] : 0.f;
    const float ydbar = atom >= 0 ? -1.f : 0.f;
    if (!wait_all(&mb_load, ph_load)) {
      tc::mbar_wait(&mb_load, ph_load);
      failed = true;
      break;
    }
    ph_load ^= 1;
    // ---- layer 1: Z1 = X W0 (+ bias), Zdot1 = U W0
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sX, 16 * kRows, 128, 32 * kRows, sW, 16 * HP, 128, 32 * HP, n.K0p / 16, id_h,
                false);
      mma_chain(tm + kColTan, sU, 16 * kRows, 128, 32 * kRows, sW, 16 * HP, 128, 32 * HP,
                n.K0p / 16, id_h, false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    {
      float av[HP], tv[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float z[16], zd[16];
        tc::tmem_ld16(tm + lane_off + c0, z);
        tc::tmem_ld16(tm + lane_off + kColTan + c0, zd);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const float th = tanh_fast(z[q]);
          av[c0 + q] = th;
          tv[c0 + q] = (1.f - th * th) * zd[q];
        }
      }
      store_act<HP>(A1, row, av, n.H1, n.K1p);
      store_tan<HP>(T1, row, tv, n.H1, n.K1p);
    }
    publish_smem();
    // ---- layer 2: Z2 = A1 W1 (+ bias), Zdot2 = T1 W1
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sA1, 16 * kRows, 128, 32 * kRows, sW + n.off_w1f, 16 * HP, 128, 32 * HP,
                n.K1p / 16, id_h, false);
      mma_chain(tm + kColTan, sT1, 16 * kRows, 128, 32 * kRows, sW + n.off_w1f, 16 * HP, 128,
                32 * HP, n.K1p / 16, id_h, false);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    {
      float av[HP], tv[HP], zb[HP], zdb[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float z[16], zd[16];
        tc::tmem_ld16(tm + lane_off + c0, z);
        tc::tmem_ld16(tm + lane_off + kColTan + c0, zd);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const float th = tanh_fast(z[q]), pv = 1.f - th * th, wq = w2[c0 + q];
          av[c0 + q] = th;
          tv[c0 + q] = pv * zd[q];
          // abar_2 = ybar w2, adotbar_2 = ydotbar w2
          zb[c0 + q] = pv * (ybar * wq) - 2.f * th * pv * zd[q] * (ydbar * wq);
          zdb[c0 + q] = pv * (ydbar * wq);
        }
      }
      store_act<HP>(A2, row, av, n.H2, n.K2p);
      store_tan<HP>(T2, row, tv, n.H2, n.K2p);
#pragma unroll
      for (int c = 0; c < HP; c += 8) {
        st8(ZB, tc::core_off(row, c, kRows), zb + c);
        st8(ZD, tc::core_off(row, c, kRows), zdb + c);
      }
      float e0[8] = {ybar, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float e1[8] = {ydbar, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float z8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      st8(D3a, tc::core_off(row, 0, kRows), e0);
      st8(D3a, tc::core_off(row, 8, kRows), z8);
      st8(D3b, tc::core_off(row, 0, kRows), e1);
      st8(D3b, tc::core_off(row, 8, kRows), z8);
    }
    publish_smem();
    // ---- abar_1 = zbar_2 W1^T, adotbar_1 = zdotbar_2 W1^T; G1, G2
    if (tid == 0) {
      tc::fence_after_sync();
      mma_chain(tm, sZB, 16 * kRows, 128, 32 * kRows, sW + n.off_w1b, 16 * HP, 128, 32 * HP,
                HP / 16, id_h, false);
      mma_chain(tm + kColTan, sZD, 16 * kRows, 128, 32 * kRows, sW + n.off_w1b, 16 * HP, 128,
                32 * HP, HP / 16, id_h, false);
      mma_chain(tm + kColG1, sA1, 128, 16 * kRows, 256, sZB, 128, 16 * kRows, 256, kRows / 16,
                id_g, gacc);
      mma_chain(tm + kColG1, sT1, 128, 16 * kRows, 256, sZD, 128, 16 * kRows, 256, kRows / 16,
                id_g, true);
      mma_chain(tm + kColG2, sA2, 128, 16 * kRows, 256, sD3a, 128, 16 * kRows, 256, kRows / 16,
                id_g2, gacc);
      mma_chain(tm + kColG2, sT2, 128, 16 * kRows, 256, sD3b, 128, 16 * kRows, 256, kRows / 16,
                id_g2, true);
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    {
      // zbar_1 = f' abar_1 + f'' zdot_1 adotbar_1 with f'' zdot_1 = -2 a_1 t_1 (tanh)
      float zb[HP], zdb[HP];
#pragma unroll
      for (int c0 = 0; c0 < HP; c0 += 16) {
        float ab[16], tb[16], a1[16], t1[16];
        tc::tmem_ld16(tm + lane_off + c0, ab);
        tc::tmem_ld16(tm + lane_off + kColTan + c0, tb);
        tc::tmem_wait_ld();
        ld8(A1, tc::core_off(row, c0, kRows), a1);
        ld8(A1, tc::core_off(row, c0 + 8, kRows), a1 + 8);
        ld8(T1, tc::core_off(row, c0, kRows), t1);
        ld8(T1, tc::core_off(row, c0 + 8, kRows), t1 + 8);
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int j = c0 + q;
          const float av = j < n.H1 ? a1[q] : 0.f, pv = 1.f - av * av;
          zb[j] = pv * ab[q] - 2.f * av * t1[q] * tb[q];
          zdb[j] = pv * tb[q];
        }
      }
#pragma unroll
      for (int c = 0; c < HP; c += 8) {
        st8(ZB, tc::core_off(row, c, kRows), zb + c);
        st8(ZD, tc::core_off(row, c, kRows), zdb + c);
      }
    }
    publish_smem();
    // ---- G0 += X^T zbar_1 + U^T zdotbar_1
    if (tid == 0) {
      tc::fence_after_sync();
      for (int mt = 0; mt < n.nmt0; mt++) {
        mma_chain(tm + kColG0 + mt * HP, sX + mt * 16 * 16 * kRows, 128, 16 * kRows, 256, sZB,
                  128, 16 * kRows, 256, kRows / 16, id_g, gacc);
        mma_chain(tm + kColG0 + mt * HP, sU + mt * 16 * 16 * kRows, 128, 16 * kRows, 256, sZD,
                  128, 16 * kRows, 256, kRows / 16, id_g, true);
      }
      tc::mma_commit(&mb_mma);
    }
    TC_WAIT(mb_mma, ph_mma);
    gacc = true;
  }
  if (!failed) {
    if (gacc) {
      flush_tan(cur_sp);
      touched |= 1ull << cur_sp;
    }
    if (tid < a.nsp) a.gflag[(int64_t)blockIdx.x * a.nsp + tid] = (int)((touched >> tid) & 1);
  }
  if (failed && tid == 0) atomicExch(a.err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tm, kTmemCols);
}

// tangents of the standardised inputs ([N][nf] atom order, the context's arithmetic) -> BF16
// tiles in the feature layout; the bias column and padding rows are zero
template <typename T>
__global__ void pack_u_kernel(const T *u, int nf, int K0p, const int32_t *tile_atoms,
                              int64_t ntiles, uint32_t x_bytes, unsigned char *out,
                              int64_t natoms) {
  const int groups = K0p / 8;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ntiles * kRows * groups) return;
  const int g = (int)(q % groups);
  const int64_t tr = q / groups;
  const int64_t t = tr / kRows;
  const int r = (int)(tr % kRows);
  const int atom = tile_atom(tile_atoms, tr, natoms);
  float v[8];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int k = g * 8 + c;
    v[c] = (atom >= 0 && k < nf) ? (float)u[(int64_t)atom * nf + k] : 0.f;
  }
  st8(out + t * (int64_t)x_bytes, tc::core_off(r, g * 8, kRows), v);
}

// ---- packing kernels ---------------------------------------------------------------------
// Features of every tile row (z-scored, bucketed rows of the context) -> BF16 core layout,
// constant 1 in column nf for real atoms; padding rows all zero.
template <typename T>
__global__ void pack_x_kernel(const T *feat, const int32_t *bpos, int nf, int K0p,
                              const int32_t *tile_atoms, int64_t ntiles, uint32_t x_bytes,
                              unsigned char *x, int64_t natoms) {
  const int groups = K0p / 8;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ntiles * kRows * groups) return;
  const int g = (int)(q % groups);
  const int64_t tr = q / groups;
  const int64_t t = tr / kRows;
  const int r = (int)(tr % kRows);
  const int atom = tile_atom(tile_atoms, tr, natoms);
  float v[8];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int k = g * 8 + c;
    float x0 = 0.f;
    if (atom >= 0) {
      if (k < nf) x0 = (float)feat[(int64_t)bpos[atom] * nf + k];
      else if (k == nf) x0 = 1.f;
    }
    v[c] = x0;
  }
  st8(x + t * (int64_t)x_bytes, tc::core_off(r, g * 8, kRows), v);
}

// The same packing for FP32 features whose width is a multiple of 4, one CTA per tile: the
// rows' feature offsets resolved once into shared memory, then every thread sweeps (row,
// 4-column chunk) items with 16-byte loads (consecutive threads, consecutive chunks of a row),
// the BF16 values placed in the tile's core-matrix layout in shared memory, and the finished
// tile written with 16-byte stores to consecutive addresses.  Same values and layout as
// pack_x_kernel.
constexpr int kPackThreads = 256;
__global__ void __launch_bounds__(kPackThreads) pack_x_tile_kernel(
    const float *feat, const int32_t *bpos, int nf, int K0p, const int32_t *tile_atoms,
    uint32_t x_bytes, unsigned char *x, int64_t natoms) {
  extern __shared__ __align__(16) unsigned char tile[];
  __shared__ int64_t rowoff[kRows];  // first feature of each row, -1 for padding rows
  const int64_t t = blockIdx.x;
  if (threadIdx.x < kRows) {
    const int atom = tile_atom(tile_atoms, t * kRows + threadIdx.x, natoms);
    rowoff[threadIdx.x] = atom >= 0 ? (int64_t)bpos[atom] * nf : -1;
  }
  __syncthreads();
  const int nq = nf / 4, nc = K0p / 4;  // feature chunks, chunks per row
  for (int it = threadIdx.x; it < kRows * nc; it += kPackThreads) {
    const int r = it / nc, c = it - r * nc;
    const int64_t ro = rowoff[r];
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ro >= 0) {
      if (c < nq) v = *reinterpret_cast<const float4 *>(feat + ro + 4 * c);
      else if (c == nq) v.x = 1.f;  // the constant input of the first layer's bias
    }
    const __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
    *reinterpret_cast<uint2 *>(tile + tc::core_off(r, 4 * c, kRows)) =
        make_uint2(*reinterpret_cast<const uint32_t *>(&lo), *reinterpret_cast<const uint32_t *>(&hi));
  }
  __syncthreads();
  uint4 *dst = reinterpret_cast<uint4 *>(x + t * (int64_t)x_bytes);
  const uint4 *src = reinterpret_cast<const uint4 *>(tile);
  for (uint32_t q = threadIdx.x; q < x_bytes / 16; q += kPackThreads) dst[q] = src[q];
}

// FP64 master parameters (reference order) -> per-species BF16 weight images + FP32 output
// layer: W0 image rows = first hidden units, columns = inputs (+ bias column nf); W1 forward
// image rows = second hidden units, columns = first (+ bias column H1); W1 reverse image rows =
// first hidden units, columns = second; W0 reverse image rows = inputs, columns = first hidden
// units; then w2[HP], b3 as floats.
template <int HP>
__global__ void pack_w_kernel(const double *p64, TcNet n, unsigned char *w) {
  const int s = blockIdx.y;
  const double *p = p64 + (int64_t)s * n.nparams;
  unsigned char *blk = w + (int64_t)s * n.w_bytes;
  const int e0 = HP * n.K0p, e1 = HP * n.K1p, e2 = HP * HP, e3 = n.K0p * HP;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < e0 + e1 + e2 + e3 + HP + 1;
       q += gridDim.x * blockDim.x) {
    if (q < e0) {
      const int u = q / n.K0p, k = q % n.K0p;
      double v = 0.0;
      if (u < n.H1) v = k < n.nf ? p[n.woff0 + k + (int64_t)n.nf * u] : (k == n.nf ? p[n.boff1 + u] : 0.0);
      *reinterpret_cast<__nv_bfloat16 *>(blk + tc::core_off(u, k, HP)) = __float2bfloat16_rn((float)v);
    } else if (q < e0 + e1) {
      const int r = q - e0, i = r / n.K1p, j = r % n.K1p;
      double v = 0.0;
      if (i < n.H2) v = j < n.H1 ? p[n.woff1 + j + (int64_t)n.H1 * i] : (j == n.H1 ? p[n.boff2 + i] : 0.0);
      *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w1f + tc::core_off(i, j, HP)) =
          __float2bfloat16_rn((float)v);
    } else if (q < e0 + e1 + e2) {
      const int r = q - e0 - e1, j = r / HP, i = r % HP;
      const double v = (j < n.H1 && i < n.H2) ? p[n.woff1 + j + (int64_t)n.H1 * i] : 0.0;
      *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w1b + tc::core_off(j, i, HP)) =
          __float2bfloat16_rn((float)v);
    } else if (q < e0 + e1 + e2 + e3) {
      // reverse image of W0 (rows = inputs, columns = first hidden units) for d out / d x
      const int r = q - e0 - e1 - e2, k = r / HP, j = r % HP;
      const double v = (k < n.nf && j < n.H1) ? p[n.woff0 + k + (int64_t)n.nf * j] : 0.0;
      *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w0b + tc::core_off(k, j, n.K0p)) =
          __float2bfloat16_rn((float)v);
    } else {
      const int i = q - e0 - e1 - e2 - e3;  // i < HP: output weights, i == HP: output bias
      float *tail = reinterpret_cast<float *>(blk + n.off_w2);
      tail[i] = i < HP ? (i < n.H2 ? (float)p[n.woff2 + i] : 0.f) : (float)p[n.boff3];
    }
  }
}

// FP64 sums of the per-CTA partials in CTA order (deterministic); parameters no kernel
// produces (the unused output-layer ww(d_L, 1) and the input-layer biases) are zero.  Every
// block also records the largest |g| of its parameters (bmax[species][block]) for the update's
// displacement limit.
constexpr int kRedThreads = 256;
constexpr int kRedSplit = 8;  // threads sharing one parameter's CTA loop

// hi + lo += v exactly up to the rounding of lo (Knuth's TwoSum on the FP32 pipe): the sums of
// FP32 partials keep 48 significant bits, more than the FP64 pipe (a 64th of the FP32 rate on
// this GPU) would be needed for, in a fixed order
__device__ __forceinline__ void df_add(float &hi, float &lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
  hi = s;
}

__global__ void __launch_bounds__(kRedThreads) tc_reduce_kernel(const float *gpart,
                                                                const int32_t *gflag, int nblk,
                                                                int nsp, TcNet n, double *grad64,
                                                                double *bmax) {
  __shared__ int list[kMaxTcBlocks];  // the CTAs that wrote a partial of this species, in order
  __shared__ unsigned char on[kMaxTcBlocks];
  __shared__ int nlist;
  __shared__ float2 part[kRedSplit][kRedThreads / kRedSplit];
  __shared__ double sh[kRedThreads / kRedSplit];
  const int s = blockIdx.y;
  // the flags of every CTA, read by all threads at once (one round of loads), then compacted
  // by one warp in CTA order (tiles are sorted by species, so a species' CTAs form a short run)
  for (int b = threadIdx.x; b < nblk; b += kRedThreads) on[b] = gflag[b * nsp + s] != 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    int cnt = 0;
    for (int b0 = 0; b0 < nblk; b0 += 32) {
      const int b = b0 + threadIdx.x;
      const bool f = b < nblk && on[b];
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (f) list[cnt + __popc(m & ((1u << threadIdx.x) - 1u))] = b;
      cnt += __popc(m);
    }
    if (threadIdx.x == 0) nlist = cnt;
  }
  __syncthreads();
  const int nl = nlist;
  // thread (r, k): parameter q = block * 32 + k, partials r, r + 8, ... of the list (loads
  // requested four at a time); the eight partial sums combined in r order
  constexpr int kq = kRedThreads / kRedSplit;
  const int k = threadIdx.x % kq, r = threadIdx.x / kq;
  const int64_t q = (int64_t)blockIdx.x * kq + k;
  float hi = 0.f, lo = 0.f;
  if (q < n.nparams && (q < n.woff3 || q >= n.boff1)) {
    const float *p = gpart + (int64_t)s * n.nparams + q;
    const int64_t stride = (int64_t)nsp * n.nparams;
    int i = r;
    for (; i + 3 * kRedSplit < nl; i += 4 * kRedSplit) {
      const float v0 = p[list[i] * stride], v1 = p[list[i + kRedSplit] * stride],
                  v2 = p[list[i + 2 * kRedSplit] * stride], v3 = p[list[i + 3 * kRedSplit] * stride];
      df_add(hi, lo, v0);
      df_add(hi, lo, v1);
      df_add(hi, lo, v2);
      df_add(hi, lo, v3);
    }
    for (; i < nl; i += kRedSplit) df_add(hi, lo, p[list[i] * stride]);
  }
  part[r][k] = make_float2(hi, lo);
  __syncthreads();
  if (threadIdx.x < kq) {
    float th = 0.f, tl = 0.f;
#pragma unroll
    for (int rr = 0; rr < kRedSplit; rr++) {
      const float2 v = part[rr][threadIdx.x];
      df_add(th, tl, v.x);
      tl = __fadd_rn(tl, v.y);
    }
    const double t = (double)th + (double)tl;
    const int64_t qq = (int64_t)blockIdx.x * kq + threadIdx.x;
    if (qq < n.nparams) grad64[(int64_t)s * n.nparams + qq] = t;
    sh[threadIdx.x] = fabs(t);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double m = 0.0;
    for (int t = threadIdx.x; t < kq; t += 32) m = fmax(m, sh[t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) bmax[(int64_t)s * gridDim.x + blockIdx.x] = m;
  }
}

// Parameter q of a species -> its places in the species' weight images (the packing of
// pack_w_kernel, one parameter at a time).
template <int HP>
__device__ __forceinline__ void write_images(const TcNet &n, unsigned char *blk, int64_t q,
                                             double v) {
  const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
  if (q >= n.woff0 && q < n.woff0 + (int64_t)n.nf * n.H1) {
    const int r = (int)(q - n.woff0), k = r % n.nf, j = r / n.nf;
    *reinterpret_cast<__nv_bfloat16 *>(blk + tc::core_off(j, k, HP)) = h;
    *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w0b + tc::core_off(k, j, n.K0p)) = h;
  } else if (q >= n.woff1 && q < n.woff1 + (int64_t)n.H1 * n.H2) {
    const int r = (int)(q - n.woff1), j = r % n.H1, i = r / n.H1;
    *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w1f + tc::core_off(i, j, HP)) = h;
    *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w1b + tc::core_off(j, i, HP)) = h;
  } else if (q >= n.woff2 && q < n.woff2 + n.H2) {
    reinterpret_cast<float *>(blk + n.off_w2)[q - n.woff2] = (float)v;
  } else if (q >= n.boff1 && q < n.boff1 + n.H1) {
    *reinterpret_cast<__nv_bfloat16 *>(blk + tc::core_off((int)(q - n.boff1), n.nf, HP)) = h;
  } else if (q >= n.boff2 && q < n.boff2 + n.H2) {
    *reinterpret_cast<__nv_bfloat16 *>(blk + n.off_w1f + tc::core_off((int)(q - n.boff2), n.H1, HP)) = h;
  } else if (q == n.boff3) {
    reinterpret_cast<float *>(blk + n.off_w2)[HP] = (float)v;
  }
}

// Steepest descent of every sub-network with the mini-batch gradient (steepdesc.F90:126-204
// after TBpnn_update's normalisation bpnn.F90:751-766, no regularisation): d = -lr g / sum(w),
// scaled to the maximal displacement when its largest component exceeds it; the new FP64
// parameter and its BF16 / FP32 image entries written in the same pass.
template <int HP>
__global__ void __launch_bounds__(kRedThreads) tc_update_kernel(double *params,
                                                                const double *grad,
                                                                const double *bmax, int nbm,
                                                                TcNet n, double inv_sumw,
                                                                double lr, double maxdisp,
                                                                unsigned char *w) {
  __shared__ double smax, sscale;
  __shared__ double wmax[kRedThreads / 32];
  const int s = blockIdx.y;
  {
    // the species' largest gradient component from the reduction's block maxima: every
    // thread's share loaded at once, then warp and block maxima
    double m = 0.0;
    for (int b = threadIdx.x; b < nbm; b += kRedThreads) m = fmax(m, bmax[(int64_t)s * nbm + b]);
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, k));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kRedThreads / 32; w++) t = fmax(t, wmax[w]);
      smax = lr * (t * inv_sumw);
      // the displacement's scale, one division per CTA (1 when within the limit: x + 1 d
      // equals x + d)
      sscale = smax <= maxdisp ? 1.0 : maxdisp / smax;
    }
  }
  __syncthreads();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n.nparams) return;
  double *x = params + (int64_t)s * n.nparams;
  const double d = -1.0 * lr * (grad[(int64_t)s * n.nparams + q] * inv_sumw);
  const double v = x[q] + sscale * d;
  x[q] = v;
  write_images<HP>(n, w + (int64_t)s * n.w_bytes, q, v);
}

// ---- autotuned launch shapes, kept per network shape for the process ----------------------
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, int> g_tune;  // (mode, nf, H1, H2, tiles/batch) -> CTAs

}  // namespace

struct BatchState {
  int B = 0, nbatch = 0, HP = 0;
  int64_t ntiles = 0;
  TcNet net{};
  std::vector<int64_t> tile0;  // [nbatch + 1] first tile of every mini-batch
  std::vector<int32_t> s0;     // [nbatch + 1] first structure of every mini-batch
  std::vector<double> sumw;    // [nbatch] datapoint weights of every mini-batch
  DBuf d_tile_sp, d_tile_atoms, d_x, d_u, d_w, d_gpart, d_gflag, d_err, d_bmax;
  int grid_fwd = 0, grid_train = 0;
  // what the tile plan was built for
  int plan_S = -1, plan_nsp = 0;
  int64_t plan_N = -1;
  std::vector<int32_t> plan_dims;
  uint64_t plan_layout = 0;  // the context's structure/species generation of the plan
  // captured epoch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double g_lr = -1.0, g_maxdisp = -1.0;
  int g_loss = -1;
  int64_t g_launches = 0;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  ~BatchState() { drop_graph(); }
};

void batch_free(BatchState *b) { delete b; }

namespace {

template <int HP> void *tc_kernel(int mode) {
  return mode == 0 ? (void *)tc_mlp_kernel<HP, 0> : (void *)tc_mlp_kernel<HP, 1>;
}
void *tc_kernel_hp(int hp, int mode) {
  switch (hp) {
    case 16: return tc_kernel<16>(mode);
    case 32: return tc_kernel<32>(mode);
    default: return tc_kernel<64>(mode);
  }
}
void *tc_jac_hp(int hp) {
  return hp == 16 ? (void *)tc_jac_kernel<16>
                  : (hp == 32 ? (void *)tc_jac_kernel<32> : (void *)tc_jac_kernel<64>);
}
void *tc_tan_hp(int hp) {
  return hp == 16 ? (void *)tc_tan_kernel<16>
                  : (hp == 32 ? (void *)tc_tan_kernel<32> : (void *)tc_tan_kernel<64>);
}

int launch_tc(fnetg_ctx *ctx, int mode, int64_t t0, int64_t t1, int grid) {
  BatchState &b = *ctx->batch;
  if (t1 <= t0) return FNETG_OK;
  TcArgs a{};
  a.net = b.net;
  a.x = b.d_x.as<unsigned char>();
  a.w = b.d_w.as<unsigned char>();
  a.tile_sp = b.d_tile_sp.as<int32_t>();
  a.tile_atoms = b.d_tile_atoms.as<int32_t>();
  a.natoms = ctx->N;
  a.t0 = t0;
  a.t1 = t1;
  a.out = ctx->d_out.as<double>();
  a.delta = ctx->d_lossgrad.as<double>();
  a.gpart = b.d_gpart.as<float>();
  a.gflag = b.d_gflag.as<int32_t>();
  a.nsp = ctx->nsp;
  a.err = b.d_err.as<int>();
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(grid, t1 - t0));
  void *k = tc_kernel_hp(b.HP, mode);
  if (mode == 0) ctx->out_fgen = ctx->out_pgen = -1;  // d_out now holds the BF16 forward
  const uint32_t smem = mode == 0 ? b.net.fm_total : b.net.sm_total;
  FNETG_CUDA(raise_smem_limit(k, smem));
  void *args[] = {&a};
  LaunchScope ls(ctx, mode == 0 ? "tc_forward" : "tc_train");
  FNETG_CUDA(cudaLaunchKernel(k, dim3(grid), dim3(kMlpThreads), args, smem, ctx->stream));
  return FNETG_OK;
}

TcArgs base_args(fnetg_ctx *ctx, int64_t t0, int64_t t1) {
  BatchState &b = *ctx->batch;
  TcArgs a{};
  a.net = b.net;
  a.x = b.d_x.as<unsigned char>();
  a.w = b.d_w.as<unsigned char>();
  a.tile_sp = b.d_tile_sp.as<int32_t>();
  a.tile_atoms = b.d_tile_atoms.as<int32_t>();
  a.natoms = ctx->N;
  a.t0 = t0;
  a.t1 = t1;
  a.out = ctx->d_out.as<double>();
  a.delta = ctx->d_lossgrad.as<double>();
  a.gpart = b.d_gpart.as<float>();
  a.gflag = b.d_gflag.as<int32_t>();
  a.nsp = ctx->nsp;
  a.err = b.d_err.as<int>();
  return a;
}

// the input Jacobian of every atom of tiles [t0, t1) into d_jacT (scaled for the force kernel)
int launch_tc_jac(fnetg_ctx *ctx, int64_t t0, int64_t t1, int grid) {
  BatchState &b = *ctx->batch;
  if (t1 <= t0) return FNETG_OK;
  TcArgs a = base_args(ctx, t0, t1);
  FNETG_CUDA(ctx->d_jacT.ensure(sizeof(float) * std::max<int64_t>(ctx->N, 1) * ctx->nf));
  a.jac = ctx->d_jacT.as<float>();
  a.zinv = ctx->d_zprec_f.as<float>() + ctx->gf.size();
  a.ng = (int)ctx->gf.size();
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(grid, t1 - t0));
  void *k = tc_jac_hp(b.HP);
  FNETG_CUDA(raise_smem_limit(k, b.net.jm_total));
  void *args[] = {&a};
  ctx->out_fgen = ctx->out_pgen = -1;
  LaunchScope ls(ctx, "tc_jacobian");
  FNETG_CUDA(cudaLaunchKernel(k, dim3(grid), dim3(kThreads), args, b.net.jm_total, ctx->stream));
  return FNETG_OK;
}

// the force-loss reverse pass over tiles [t0, t1) (packed tangents in the batch state)
int launch_tc_tan(fnetg_ctx *ctx, int64_t t0, int64_t t1, int grid) {
  BatchState &b = *ctx->batch;
  if (t1 <= t0) return FNETG_OK;
  TcArgs a = base_args(ctx, t0, t1);
  a.u = b.d_u.as<unsigned char>();
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(grid, t1 - t0));
  void *k = tc_tan_hp(b.HP);
  FNETG_CUDA(raise_smem_limit(k, b.net.tm_total));
  void *args[] = {&a};
  LaunchScope ls(ctx, "tc_tangent");
  FNETG_CUDA(cudaLaunchKernel(k, dim3(grid), dim3(kThreads), args, b.net.tm_total, ctx->stream));
  return FNETG_OK;
}

int launch_reduce(fnetg_ctx *ctx, int nblk) {
  BatchState &b = *ctx->batch;
  dim3 grid(ceil_div(b.net.nparams, kRedThreads / kRedSplit), ctx->nsp);
  LaunchScope ls(ctx, "tc_reduce");
  tc_reduce_kernel<<<grid, kRedThreads, 0, ctx->stream>>>(
      b.d_gpart.as<float>(), b.d_gflag.as<int32_t>(), nblk, ctx->nsp, b.net,
      ctx->d_grad64.as<double>(), b.d_bmax.as<double>());
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

int launch_pack_w(fnetg_ctx *ctx) {
  BatchState &b = *ctx->batch;
  dim3 grid(64, ctx->nsp);
  LaunchScope ls(ctx, "tc_pack");
  switch (b.HP) {
    case 16: pack_w_kernel<16><<<grid, 256, 0, ctx->stream>>>(ctx->d_params64.as<double>(), b.net, b.d_w.as<unsigned char>()); break;
    case 32: pack_w_kernel<32><<<grid, 256, 0, ctx->stream>>>(ctx->d_params64.as<double>(), b.net, b.d_w.as<unsigned char>()); break;
    default: pack_w_kernel<64><<<grid, 256, 0, ctx->stream>>>(ctx->d_params64.as<double>(), b.net, b.d_w.as<unsigned char>()); break;
  }
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

// one mini-batch: forward, loss (the reference's loss gradients per atom), reverse pass with
// weight gradients, FP64 reduction; with update: steepest descent and the new BF16 weights
int batch_step(fnetg_ctx *ctx, int k, int loss, bool update, double lr, double maxdisp) {
  BatchState &b = *ctx->batch;
  int rc = launch_tc(ctx, 0, b.tile0[k], b.tile0[k + 1], b.grid_fwd);
  if (rc) return rc;
  rc = launch_loss_range(ctx, b.s0[k], b.s0[k + 1] - b.s0[k], loss);
  if (rc) return rc;
  rc = launch_tc(ctx, 1, b.tile0[k], b.tile0[k + 1], b.grid_train);
  if (rc) return rc;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(b.grid_train, b.tile0[k + 1] - b.tile0[k]));
  rc = launch_reduce(ctx, nblk);
  if (rc) return rc;
  if (!update) return FNETG_OK;
  dim3 grid(ceil_div(b.net.nparams, kRedThreads), ctx->nsp);
  LaunchScope ls(ctx, "tc_update");
  void *kern = b.HP == 16 ? (void *)tc_update_kernel<16>
                          : (b.HP == 32 ? (void *)tc_update_kernel<32> : (void *)tc_update_kernel<64>);
  double *p64 = ctx->d_params64.as<double>();
  const double *g64 = ctx->d_grad64.as<double>();
  const double *bm = b.d_bmax.as<double>();
  int nbm = ceil_div(b.net.nparams, kRedThreads / kRedSplit);
  TcNet net = b.net;
  double inv = 1.0 / b.sumw[k];
  unsigned char *wimg = b.d_w.as<unsigned char>();
  void *args[] = {&p64, &g64, &bm, &nbm, &net, &inv, &lr, &maxdisp, &wimg};
  FNETG_CUDA(cudaLaunchKernel(kern, grid, dim3(kRedThreads), args, 0, ctx->stream));
  return FNETG_OK;
}

int check_err(fnetg_ctx *ctx) {
  int e = 0;
  FNETG_CUDA(cudaMemcpyAsync(&e, ctx->batch->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  FNETG_CHECK(e == 0, FNETG_E_TIMEOUT, "tensor-core kernel: a bounded wait gave up");
  return FNETG_OK;
}

// Time the candidate CTA counts of one stage on mini-batch 0 and keep the fastest.
int autotune(fnetg_ctx *ctx, int mode, int loss) {
  BatchState &b = *ctx->batch;
  const int64_t tiles = b.tile0[1] - b.tile0[0];
  const auto key = std::make_tuple(mode, b.net.nf, b.net.H1, b.net.H2, (int)tiles);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      (mode == 0 ? b.grid_fwd : b.grid_train) = it->second;
      return FNETG_OK;
    }
  }
  const int sms = num_sms();
  // the forward kernel's plan fits two CTAs on an SM; the training kernel's one
  const int gmax = mode == 0 ? 2 * sms : sms;
  std::vector<int> cand = {sms, sms / 2, sms / 4, (int)((tiles + 3) / 4), (int)((tiles + 5) / 6),
                           (int)((tiles + 7) / 8)};
  if (mode == 0) cand.insert(cand.begin(), {2 * sms, (int)((tiles + 1) / 2)});
  int best = sms;
  float best_ms = 1e30f;
  if (mode == 1) {  // the reverse pass reads the forward's loss gradients
    int rc = launch_tc(ctx, 0, b.tile0[0], b.tile0[1], sms);
    if (rc) return rc;
    rc = launch_loss_range(ctx, b.s0[0], b.s0[1] - b.s0[0], loss);
    if (rc) return rc;
  }
  for (int g : cand) {
    if (g < 1 || g > gmax) continue;
    float ms = 0.f;
    for (int rep = 0; rep < 3; rep++) {
      FNETG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
      int rc = launch_tc(ctx, mode, b.tile0[0], b.tile0[1], g);
      if (rc) return rc;
      if (mode == 1) {
        // the training stage is timed with the reduction of its per-CTA partials, whose
        // cost grows with the CTA count
        rc = launch_reduce(ctx, (int)std::max<int64_t>(1, std::min<int64_t>(g, tiles)));
        if (rc) return rc;
      }
      FNETG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
      FNETG_CUDA(cudaEventSynchronize(ctx->ev1));
      float t = 0.f;
      FNETG_CUDA(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
      ms = rep == 0 ? t : std::min(ms, t);
    }
    if (ms < best_ms) {
      best_ms = ms;
      best = g;
    }
  }
  int rc = check_err(ctx);
  if (rc) return rc;
  (mode == 0 ? b.grid_fwd : b.grid_train) = best;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  return FNETG_OK;
}

int ensure_tuned(fnetg_ctx *ctx, int loss) {
  BatchState &b = *ctx->batch;
  if (b.grid_fwd <= 0) {
    int rc = autotune(ctx, 0, loss);
    if (rc) return rc;
  }
  if (b.grid_train <= 0) {
    int rc = autotune(ctx, 1, loss);
    if (rc) return rc;
  }
  return FNETG_OK;
}

template <typename T>
int pack_features(fnetg_ctx *ctx) {
  BatchState &b = *ctx->batch;
  const int64_t total = b.ntiles * kRows * (b.net.K0p / 8);
  LaunchScope ls(ctx, "tc_pack");
  if (sizeof(T) == 4 && b.net.nf % 4 == 0) {
    const void *k = (const void *)pack_x_tile_kernel;
    FNETG_CUDA(raise_smem_limit(k, b.net.x_bytes));
    const float *f = ctx->d_feat.as<float>();
    const int32_t *bp = ctx->d_bpos.as<int32_t>(), *ta = b.d_tile_atoms.as<int32_t>();
    int nf = b.net.nf, K0p = b.net.K0p;
    uint32_t xb = b.net.x_bytes;
    unsigned char *x = b.d_x.as<unsigned char>();
    int64_t natoms = ctx->N;
    void *args[] = {&f, &bp, &nf, &K0p, &ta, &xb, &x, &natoms};
    FNETG_CUDA(cudaLaunchKernel(k, dim3((unsigned)b.ntiles), dim3(kPackThreads), args, b.net.x_bytes,
                                ctx->stream));
    return FNETG_OK;
  }
  pack_x_kernel<T><<<ceil_div(total, 256), 256, 0, ctx->stream>>>(
      ctx->d_feat.as<T>(), ctx->d_bpos.as<int32_t>(), b.net.nf, b.net.K0p,
      b.d_tile_atoms.as<int32_t>(), b.ntiles, b.net.x_bytes, b.d_x.as<unsigned char>(), ctx->N);
  FNETG_CUDA(cudaGetLastError());
  return FNETG_OK;
}

}  // namespace

// The full-batch training gradient (every tile of every mini-batch in one launch per stage)
// with the tensor-core network passes, for fnetg_train_gradients / fnetg_train_iteration:
//   energies only: forward, loss, reverse pass with weight gradients, FP64 reduction;
//   with a force term: forward + input Jacobian (one kernel), loss, analytical forces from that
//   Jacobian (FP32 kernel), the force term and its input tangents (FP32), the tangent reverse
//   pass, FP64 reduction.
int run_batch_gradients(fnetg_ctx *ctx, int loss) {
  FNETG_CHECK(ctx->batch != nullptr, FNETG_E_INVALID, "tensor-core training: no batch setup");
  BatchState &b = *ctx->batch;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(num_sms(), b.ntiles));
  int rc = launch_pack_w(ctx);  // the parameters may have moved since the last images
  if (rc) return rc;
  FNETG_CUDA(ctx->d_grad64.ensure(sizeof(double) * ctx->nsp * ctx->nparams));
  if (ctx->fl_weight > 0.0) {
    FNETG_CHECK(ctx->prec == FNETG_FP32 && ctx->nb_valid && ctx->zprec_valid, FNETG_E_INVALID,
                "tensor-core force loss: FP32 context with neighbour list and z-scored features");
    FNETG_CHECK(b.net.tm_total <= 227 * 1024, FNETG_E_UNSUPPORTED,
                "tensor-core force loss: tile buffers exceed shared memory (inputs too wide)");
    rc = launch_tc_jac(ctx, 0, b.ntiles, grid);
    if (rc) return rc;
    rc = launch_loss_range(ctx, 0, ctx->S, loss);
    if (rc) return rc;
    rc = launch_loss_reduce(ctx);
    if (rc) return rc;
    ctx->jac_ready = true;
    rc = run_forces(ctx);
    ctx->jac_ready = false;
    if (rc) return rc;
    rc = run_force_loss_terms(ctx);
    if (rc) return rc;
    FNETG_CUDA(b.d_u.ensure((size_t)b.ntiles * b.net.x_bytes));
    {
      const int64_t total = b.ntiles * kRows * (b.net.K0p / 8);
      LaunchScope ls(ctx, "tc_pack");
      pack_u_kernel<float><<<ceil_div(total, 256), 256, 0, ctx->stream>>>(
          ctx->d_fl_u.as<float>(), ctx->nf, b.net.K0p, b.d_tile_atoms.as<int32_t>(), b.ntiles,
          b.net.x_bytes, b.d_u.as<unsigned char>(), ctx->N);
      FNETG_CUDA(cudaGetLastError());
    }
    rc = launch_tc_tan(ctx, 0, b.ntiles, grid);
    if (rc) return rc;
  } else {
    rc = launch_tc(ctx, 0, 0, b.ntiles, 2 * num_sms());  // two forward CTAs fit on an SM
    if (rc) return rc;
    rc = launch_loss_range(ctx, 0, ctx->S, loss);
    if (rc) return rc;
    rc = launch_loss_reduce(ctx);
    if (rc) return rc;
    rc = launch_tc(ctx, 1, 0, b.ntiles, grid);
    if (rc) return rc;
  }
  return launch_reduce(ctx, grid);
}

FNETG_CHECK_READER(check_site_batch)

}  // namespace fnetg

using namespace fnetg;

extern "C" {

int fnetg_batch_setup(fnetg_ctx *ctx, int32_t batch_structures) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(batch_structures >= 1, FNETG_E_INVALID, "batch_setup: batch size must be >= 1");
  FNETG_CHECK(ctx->net_set, FNETG_E_INVALID, "batch_setup: no network");
  FNETG_CHECK(ctx->feats_valid, FNETG_E_INVALID, "batch_setup: no features computed");
  FNETG_CHECK(ctx->nf == ctx->dims[0], FNETG_E_SHAPE, "batch_setup: network input width");
  FNETG_CHECK(ctx->nlayer == 4 && ctx->dims[3] == 1 && ctx->act == FNETG_ACT_TANH &&
                  (!ctx->targets_set || (ctx->ngt == 1 && ctx->nat == 0)),
              FNETG_E_UNSUPPORTED,
              "batch_setup: the tensor-core form takes two tanh hidden layers, one output and "
              "(for training) one global target");
  const int H = std::max(ctx->dims[1], ctx->dims[2]);
  FNETG_CHECK(H <= 64 && ctx->dims[0] + 1 <= 2 * kRows - 16, FNETG_E_UNSUPPORTED,
              "batch_setup: hidden layers of at most 64 units and at most 239 inputs");
  FNETG_CHECK(ctx->nsp <= 64, FNETG_E_UNSUPPORTED, "batch_setup: at most 64 sub-networks");
  if (!ctx->batch) ctx->batch = new BatchState();
  BatchState &b = *ctx->batch;
  if (b.B == batch_structures && b.plan_S == ctx->S && b.plan_N == ctx->N &&
      b.plan_dims == ctx->dims && b.plan_nsp == ctx->nsp && b.plan_layout == ctx->layout_gen) {
    // same structures, species, network shape and batch size: the tile plan, the graph and the
    // tuned launch shapes stay; only the features and weights are packed again
    int rc = ctx->prec == FNETG_FP64 ? pack_features<double>(ctx) : pack_features<float>(ctx);
    if (rc) return rc;
    return launch_pack_w(ctx);
  }
  b.drop_graph();
  b.plan_S = -1;
  b.HP = H <= 16 ? 16 : (H <= 32 ? 32 : 64);
  b.net = b.HP == 16 ? make_net<16>(ctx) : (b.HP == 32 ? make_net<32>(ctx) : make_net<64>(ctx));
  FNETG_CHECK(b.net.jm_total <= 227 * 1024, FNETG_E_UNSUPPORTED,
              "batch_setup: tile buffers exceed shared memory");
  b.B = batch_structures;
  const int S = ctx->S;
  b.nbatch = (S + b.B - 1) / b.B;
  b.tile0.assign(1, 0);
  b.s0.assign(1, 0);
  b.sumw.clear();
  std::vector<int32_t> tsp, tatoms;
  std::vector<int32_t> w(S, 1);  // datapoint weights (1 for predictions without targets)
  if (S > 0 && ctx->targets_set)
    FNETG_CUDA(copy_sync(ctx, w.data(), ctx->d_w.p, sizeof(int32_t) * S, cudaMemcpyDeviceToHost));
  std::vector<std::vector<int32_t>> rows(ctx->nsp);
  for (int k = 0; k < b.nbatch; k++) {
    const int sa = k * b.B, se = std::min(S, sa + b.B);
    double sw = 0.0;
    for (int s = sa; s < se; s++) sw += (double)w[s];
    for (auto &r : rows) r.clear();
    for (int64_t at = ctx->h_off[sa]; at < ctx->h_off[se]; at++)
      rows[ctx->h_species[at]].push_back((int32_t)at);
    for (int sp = 0; sp < ctx->nsp; sp++)
      for (size_t r0 = 0; r0 < rows[sp].size(); r0 += kRows) {
        tsp.push_back(sp);
        for (int r = 0; r < kRows; r++)
          tatoms.push_back(r0 + r < rows[sp].size() ? rows[sp][r0 + r] : -1);
      }
    b.tile0.push_back((int64_t)tsp.size());
    b.s0.push_back(se);
    b.sumw.push_back(sw);
    FNETG_CHECK(sw > 0.0, FNETG_E_INVALID, "batch_setup: a mini-batch has zero total weight");
  }
  b.ntiles = (int64_t)tsp.size();
  FNETG_CHECK(b.ntiles > 0, FNETG_E_INVALID, "batch_setup: no atoms");
  FNETG_CUDA(b.d_tile_sp.ensure(sizeof(int32_t) * b.ntiles));
  FNETG_CUDA(b.d_tile_atoms.ensure(sizeof(int32_t) * b.ntiles * kRows));
  FNETG_CUDA(copy_sync(ctx, b.d_tile_sp.p, tsp.data(), sizeof(int32_t) * b.ntiles, cudaMemcpyHostToDevice));
  FNETG_CUDA(copy_sync(ctx, b.d_tile_atoms.p, tatoms.data(), sizeof(int32_t) * tatoms.size(),
                        cudaMemcpyHostToDevice));
  FNETG_CUDA(b.d_x.ensure((size_t)b.ntiles * b.net.x_bytes));
  FNETG_CUDA(b.d_w.ensure((size_t)ctx->nsp * b.net.w_bytes));
  const int maxgrid = num_sms();
  FNETG_CUDA(b.d_gpart.ensure(sizeof(float) * (size_t)maxgrid * ctx->nsp * b.net.nparams));
  FNETG_CUDA(b.d_gflag.ensure(sizeof(int32_t) * (size_t)maxgrid * ctx->nsp));
  FNETG_CUDA(b.d_bmax.ensure(sizeof(double) * (size_t)ctx->nsp *
                             ceil_div(b.net.nparams, kRedThreads / kRedSplit)));
  FNETG_CUDA(b.d_err.ensure(sizeof(int)));
  FNETG_CUDA(cudaMemsetAsync(b.d_err.p, 0, sizeof(int), ctx->stream));
  FNETG_CUDA(ctx->d_out.ensure(sizeof(double) * std::max<int64_t>(ctx->N, 1)));
  FNETG_CUDA(ctx->d_lossgrad.ensure(sizeof(double) * std::max<int64_t>(ctx->N, 1)));
  FNETG_CUDA(ctx->d_losspart.ensure(sizeof(double) * 2 * std::max(S, 1)));
  FNETG_CUDA(ctx->d_scalars.ensure(sizeof(double) * 16));
  FNETG_CUDA(ctx->d_grad64.ensure(sizeof(double) * ctx->nsp * ctx->nparams));
  int rc = ctx->prec == FNETG_FP64 ? pack_features<double>(ctx) : pack_features<float>(ctx);
  if (rc) return rc;
  rc = launch_pack_w(ctx);
  if (rc) return rc;
  b.grid_fwd = b.grid_train = 0;
  b.plan_S = ctx->S;
  b.plan_N = ctx->N;
  b.plan_dims = ctx->dims;
  b.plan_nsp = ctx->nsp;
  b.plan_layout = ctx->layout_gen;
  FNETG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FNETG_OK;
}

int fnetg_batch_info(fnetg_ctx *ctx, int32_t *nbatch, int64_t *ntiles, int32_t *ctas_forward,
                     int32_t *ctas_train) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  if (nbatch) *nbatch = ctx->batch->nbatch;
  if (ntiles) *ntiles = ctx->batch->ntiles;
  if (ctas_forward) *ctas_forward = ctx->batch->grid_fwd;
  if (ctas_train) *ctas_train = ctx->batch->grid_train;
  return FNETG_OK;
}

int fnetg_batch_gradients(fnetg_ctx *ctx, int32_t batch, int32_t loss, double *grad,
                          double *atomic_out) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->targets_set, FNETG_E_INVALID, "batch_gradients: no targets");
  BatchState &b = *ctx->batch;
  FNETG_CHECK(batch >= 0 && batch < b.nbatch, FNETG_E_INVALID, "batch_gradients: batch index");
  FNETG_CHECK(loss >= 0 && loss <= 3, FNETG_E_INVALID, "loss code");
  int rc = ensure_tuned(ctx, loss);
  if (rc) return rc;
  rc = batch_step(ctx, batch, loss, false, 0.0, 0.0);
  if (rc) return rc;
  rc = check_err(ctx);
  if (rc) return rc;
  if (grad)
    FNETG_CUDA(copy_sync(ctx, grad, ctx->d_grad64.p, sizeof(double) * ctx->nsp * ctx->nparams,
                          cudaMemcpyDeviceToHost));
  if (atomic_out) {
    const int64_t a0 = ctx->h_off[b.s0[batch]], a1 = ctx->h_off[b.s0[batch + 1]];
    if (a1 > a0)
      FNETG_CUDA(copy_sync(ctx, atomic_out, ctx->d_out.as<double>() + a0,
                            sizeof(double) * (a1 - a0), cudaMemcpyDeviceToHost));
  }
  return FNETG_OK;
}

int fnetg_batch_epoch(fnetg_ctx *ctx, int32_t loss, double learning_rate, double max_disp,
                      double *loss_out) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  FNETG_CHECK(ctx->targets_set, FNETG_E_INVALID, "batch_epoch: no targets");
  BatchState &b = *ctx->batch;
  FNETG_CHECK(loss >= 0 && loss <= 3, FNETG_E_INVALID, "loss code");
  FNETG_CHECK(learning_rate > 0.0 && max_disp > 0.0, FNETG_E_INVALID,
              "batch_epoch: learning rate and maximal displacement must be > 0");
  int rc = ensure_tuned(ctx, loss);
  if (rc) return rc;
  if (ctx->prof) {
    // per-kernel timing requested: the same launches eagerly, each with its CUDA events
    for (int k = 0; k < b.nbatch; k++) {
      rc = batch_step(ctx, k, loss, true, learning_rate, max_disp);
      if (rc) return rc;
    }
    rc = launch_loss_reduce(ctx);
    if (rc) return rc;
    if (loss_out) {
      FNETG_CUDA(cudaMemcpyAsync(loss_out, ctx->d_scalars.p, sizeof(double),
                                 cudaMemcpyDeviceToHost, ctx->stream));
      return check_err(ctx);
    }
    return FNETG_OK;
  }
  if (!b.exec || b.g_lr != learning_rate || b.g_maxdisp != max_disp || b.g_loss != loss) {
    b.drop_graph();
    // capture every mini-batch step and the epoch loss as one graph (no timing events inside)
    const bool prof = ctx->prof;
    ctx->prof = false;
    const int64_t l0 = ctx->launches;
    FNETG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int crc = FNETG_OK;
    for (int k = 0; k < b.nbatch && crc == FNETG_OK; k++)
      crc = batch_step(ctx, k, loss, true, learning_rate, max_disp);
    if (crc == FNETG_OK) crc = launch_loss_reduce(ctx);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->prof = prof;
    b.g_launches = ctx->launches - l0;
    ctx->launches = l0;
    if (crc) {
      if (g) cudaGraphDestroy(g);
      return crc;
    }
    FNETG_CUDA(e);
    b.graph = g;
    FNETG_CUDA(cudaGraphInstantiate(&b.exec, b.graph, 0));
    b.g_lr = learning_rate;
    b.g_maxdisp = max_disp;
    b.g_loss = loss;
  }
  {
    LaunchScope ls(ctx, "tc_epoch");
    FNETG_CUDA(cudaGraphLaunch(b.exec, ctx->stream));
  }
  ctx->launches += b.g_launches - 1;
  if (loss_out) {
    FNETG_CUDA(cudaMemcpyAsync(loss_out, ctx->d_scalars.p, sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
    return check_err(ctx);
  }
  return FNETG_OK;
}

int fnetg_batch_predict(fnetg_ctx *ctx, double *atomic_out, double *global_out) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  BatchState &b = *ctx->batch;
  int rc = ensure_tuned(ctx, 0);
  if (rc) return rc;
  rc = launch_tc(ctx, 0, 0, b.ntiles, 2 * num_sms());
  if (rc) return rc;
  if (global_out && ctx->S > 0) {
    FNETG_CUDA(ctx->d_gsum.ensure(sizeof(double) * ctx->S));
    LaunchScope ls(ctx, "struct_sum");
    struct_sum_kernel<<<ceil_div(ctx->S, 128), 128, 0, ctx->stream>>>(
        ctx->d_out.as<double>(), ctx->d_off.as<int64_t>(), ctx->S, 1, ctx->d_gsum.as<double>());
    FNETG_CUDA(cudaGetLastError());
  }
  if (atomic_out && ctx->N > 0)
    FNETG_CUDA(cudaMemcpyAsync(atomic_out, ctx->d_out.p, sizeof(double) * ctx->N,
                               cudaMemcpyDeviceToHost, ctx->stream));
  if (global_out && ctx->S > 0)
    FNETG_CUDA(cudaMemcpyAsync(global_out, ctx->d_gsum.p, sizeof(double) * ctx->S,
                               cudaMemcpyDeviceToHost, ctx->stream));
  if (atomic_out || global_out) return check_err(ctx);
  return FNETG_OK;
}

int fnetg_batch_forces(fnetg_ctx *ctx, double *global_out, double *forces_out) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  BatchState &b = *ctx->batch;
  FNETG_CHECK(ctx->prec == FNETG_FP32 && ctx->nb_valid && ctx->zprec_valid, FNETG_E_INVALID,
              "batch_forces: FP32 context with neighbour list and z-scored features");
  FNETG_CHECK(b.plan_S == ctx->S && b.plan_N == ctx->N, FNETG_E_INVALID,
              "batch_forces: the structures changed since fnetg_batch_setup");
  // forward and input Jacobian of every tile in one launch (a CTA per tile up to the SM count)
  int rc = launch_tc_jac(ctx, 0, b.ntiles, (int)std::min<int64_t>(num_sms(), b.ntiles));
  if (rc) return rc;
  ctx->jac_ready = true;
  rc = run_forces(ctx);
  ctx->jac_ready = false;
  if (rc) return rc;
  rc = check_err(ctx);
  if (rc) return rc;
  if (global_out && ctx->S > 0) {
    FNETG_CUDA(ctx->d_gsum.ensure(sizeof(double) * ctx->S));
    {
      LaunchScope ls(ctx, "struct_sum");
      struct_sum_kernel<<<ceil_div(ctx->S, 128), 128, 0, ctx->stream>>>(
          ctx->d_out.as<double>(), ctx->d_off.as<int64_t>(), ctx->S, 1, ctx->d_gsum.as<double>());
      FNETG_CUDA(cudaGetLastError());
    }
    FNETG_CUDA(copy_sync(ctx, global_out, ctx->d_gsum.p, sizeof(double) * ctx->S,
                          cudaMemcpyDeviceToHost));
  }
  if (forces_out && ctx->N > 0)
    FNETG_CUDA(copy_sync(ctx, forces_out, ctx->d_forces.p, sizeof(double) * ctx->N * 3,
                          cudaMemcpyDeviceToHost));
  return FNETG_OK;
}

int fnetg_batch_train_bf16(fnetg_ctx *ctx, int32_t on) {
  if (!ctx) return FNETG_E_INVALID;
  FNETG_CHECK(!on || ctx->batch != nullptr, FNETG_E_INVALID,
              "batch_train_bf16: call fnetg_batch_setup first");
  ctx->batch_train = on != 0;
  return FNETG_OK;
}

int fnetg_batch_sync_params(fnetg_ctx *ctx) {
  if (!ctx || !ctx->batch) return FNETG_E_INVALID;
  int rc = launch_pack_w(ctx);
  if (rc) return rc;
  return run_params_to_compute(ctx);
}

}  // extern "C"

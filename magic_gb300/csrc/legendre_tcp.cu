// Persistent, warp-specialized tensor-core Legendre sums (3xBF16 split
// products, fp32 accumulation in tensor memory) for the radial loop's
// batched transforms.
//
// Two kernels per transform:
//  1. a pack kernel splits the data operand once into 3xBF16 tiles in the
//     exact shared-memory image of the MMA's K-major, 128-byte-swizzled
//     operand (synthesis: spectra with their operator applied, one image per
//     (m, parity, 64-degree chunk, column tile); analysis: the ES and EA half
//     spectra, one image each per (m, 64-colatitude chunk, column tile)).
//     One CTA builds the two tiles that share its input (both parities of a
//     128-degree chunk; the ES and EA tiles of 64 colatitudes) and writes them
//     with bulk copies.
//  2. one persistent CTA per SM takes output tiles from a global counter
//        synthesis tile = (m, parity, 128 colatitudes, 32 complex columns)
//        analysis tile  = (m, parity, 128 degrees of that parity, 32 complex columns)
//     with three roles:
//        warp 0      bulk-copy loader of table tiles (A ring) and data tiles (B ring)
//        warp 1      tcgen05.mma issuer (one thread)
//        warps 2..9  epilogue: two warps per TMEM lane quadrant, each draining
//                    half of the columns; the accumulators are summed into
//                    registers and released before the outputs are computed
//
// Split products: the three splits of a data tile lie one after the other
// (hi, mid, lo: 64 rows each), so one MMA with N = 192 multiplies a table
// split by all three.  Per table and K step:
//     A_hi  x [B_hi | B_mid | B_lo]  ->  [C0 | C1 | C2]   (N = 192)
//     A_mid x [B_hi | B_mid]         ->       [C1 | C2]   (N = 128)
//     A_lo  x [B_hi]                 ->            [C2]   (N = 64)
// C0 = hi*hi, C1 the 2^-8-order and C2 the 2^-16-order cross products, each
// accumulated apart in fp32 and summed (C2 + C1) + C0 in the epilogue.
// Hand-offs use full/empty mbarriers; every wait is bounded and a wait that
// gives up sets the device error word.
#include <algorithm>
#include <type_traits>
#include <vector>
#include <cuda_bf16.h>
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"
#include "tc_ptx.cuh"
#include "tc_build.cuh"

namespace {

constexpr int kNC = 64;  // real data columns per tile (32 complex)

// CTAs per SM: the scalar kernels (one table, 192 accumulator columns) run two
// CTAs per SM with 256 TMEM columns each, so that one CTA's MMA thread issues
// while the other's waits for its operands or commits; the vector kernels (two
// tables, 384 accumulator columns) need all 512 columns and run one.
// The TF32 vector kernels (twice the MMA instructions of 3xBF16 per chunk) have
// two MMA threads (warp 1 and warp 10), one per table (P and dP): each waits for
// the same operands and issues the MMAs of its own table, so one thread's
// waits, fences and commits overlap the other's MMAs (7% faster there; the
// 3xBF16 synthesis measured 4% slower with two, so it keeps one).
template <bool VEC, bool TF32>
struct Occ {
  static constexpr int CPS = VEC ? 1 : 2;
  static constexpr int TCOLS = 512 / CPS;
  static constexpr int NISS = (VEC && TF32) ? 2 : 1;  // MMA threads
  static constexpr int XTRA = NISS == 2 ? 32 : 0;      // threads beyond kThreads (the second MMA warp)
};

// ring depths: A = one table split of one K tile (NT x 16 KB per slot), B = data
// tiles (24 KB, 32 KB with TF32).  Two scalar CTAs share an SM's shared memory,
// so their rings are shallower; a vector CTA's A ring is as deep as shared
// memory allows with the TF32 data tiles.
template <bool VEC, bool INV, bool TF32>
struct Rings {
  static constexpr int NA = VEC ? (INV ? 4 : 3) : (TF32 ? 2 : 3);
  static constexpr int NB = 2;
};

// Split format of the tensor-core form.  TF32 = false: 3 bf16 splits, one K
// tile of 64 per chunk, kind::f16.  TF32 = true: 2 tf32 splits (hi, lo), two K
// tiles of 32 per chunk, kind::tf32, products hi*hi, hi*lo, lo*hi.
template <bool TF32>
struct Form {
  static constexpr int SPA = TF32 ? 2 : 3;            // table splits
  static constexpr int KT = TF32 ? 2 : 1;             // K tiles per 64-wide chunk
  static constexpr int AUSES = SPA * KT;              // A-ring uses per chunk
  static constexpr int BPC = TF32 ? 4 : 3;            // 16 KB table blocks per chunk
  static constexpr int NACCS = TF32 ? 2 : 3;          // accumulators per table
  static constexpr uint32_t OPSZ = DataTile<TF32, kNC>::bytes;  // data operand per chunk
};

constexpr int kThreads = 320;     // 10 warps
constexpr int kEpiThreads = 256;  // warps 2..9
constexpr int kPackThreads = 256;

__device__ __forceinline__ unsigned char* align1k(unsigned char* p) {
  return (unsigned char*)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

// consumer waits for "full" with the round's parity, producer waits for
// "empty" with the opposite parity (an empty ring passes at once)
__device__ __forceinline__ bool wait_full(uint64_t* bar, uint32_t use, uint32_t ring) {
  return tc::mbar_wait(bar, (use / ring) & 1u);
}
__device__ __forceinline__ bool wait_empty(uint64_t* bar, uint32_t use, uint32_t ring) {
  return tc::mbar_wait(bar, ((use / ring) & 1u) ^ 1u);
}

// The loader's last copies (one per ring slot) have landed: nothing writes
// shared memory after the CTA exits, also when a consumer gave up early.
template <int N>
__device__ __forceinline__ void drain_copies(uint64_t* full, uint32_t use) {
  for (uint32_t u = use > N ? use - N : 0; u < use; ++u) wait_full(&full[u % N], u, N);
}

// Dynamic tile schedule: the loader thread takes tile indices from a global
// counter and publishes them, in order, through a small shared-memory ring
// that the MMA thread and the epilogue threads consume (-1 ends the list).
constexpr int kNTR = 4;
struct TileRing {
  int* idx;
  uint64_t* full;   // count 1 (the loader)
  uint64_t* empty;  // count 1 + kEpiThreads (MMA thread and epilogue threads)
};
__device__ __forceinline__ bool ring_push(const TileRing& R, uint32_t& use, int ix) {
  const uint32_t slot = use % kNTR;
  if (!wait_empty(&R.empty[slot], use, kNTR)) return false;
  R.idx[slot] = ix;
  tc::mbar_arrive(&R.full[slot]);
  ++use;
  return true;
}
__device__ __forceinline__ bool ring_pop(const TileRing& R, uint32_t& use, int& ix) {
  const uint32_t slot = use % kNTR;
  if (!wait_full(&R.full[slot], use, kNTR)) return false;
  ix = R.idx[slot];
  tc::mbar_arrive(&R.empty[slot]);
  ++use;
  return true;
}

// Issue the MMAs of A-ring use `u` of a chunk (tables tb0 <= tb < tb1 of NT)
// against the stacked data splits; D holds NT accumulator groups of
// NACCS*kNC columns.
//  bf16 (u = split):  A_hi x [B_hi|B_mid|B_lo] -> [C0|C1|C2],  A_mid x [B_hi|B_mid]
//                     -> [C1|C2],  A_lo x B_hi -> C2   (K = 16 per MMA, 4 per tile)
//  tf32 (u = 2*K tile + split):  A_hi x [B_hi|B_lo] -> [C0|C1],  A_lo x B_hi -> C1
//                     (K = 8 per MMA, 4 per 32-wide K tile)
// nk: K rows of the chunk that hold degrees of the order (synthesis; 64 in
// the analysis): K steps past them multiply zero rows and are skipped.
template <int NT, bool TF32>
__device__ __forceinline__ void issue_use(uint32_t acc, const unsigned char* A, const unsigned char* B,
                                          int u, bool first_chunk, uint32_t bstride_tb, int tb0, int tb1,
                                          int nk = 64) {
  constexpr int NACCS = Form<TF32>::NACCS;
  const uint64_t a0 = tc::sw128_desc(tc::smem_u32(A));
  const uint64_t bd0 = tc::sw128_desc(tc::smem_u32(B));
  if constexpr (!TF32) {
    constexpr uint32_t ID3 = tc::idesc_bf16(128, 3 * kNC), ID2 = tc::idesc_bf16(128, 2 * kNC),
                       ID1 = tc::idesc_bf16(128, kNC);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks)
#pragma unroll
      for (int tb = 0; tb < NT; ++tb) {
        if (tb < tb0 || tb >= tb1) continue;  // tables of the other MMA thread
        if (16 * ks >= nk) continue;
        const uint32_t d = acc + (uint32_t)(tb * NACCS * kNC);
        const uint64_t ad = a0 + (uint64_t)((tb * 16384 + ks * 32) >> 4);
        const uint64_t bd = bd0 + (uint64_t)((tb * bstride_tb + ks * 32) >> 4);
        if (u == 0) tc::mma_bf16(d, ad, bd, ID3, (!first_chunk || ks) ? 1u : 0u);
        else if (u == 1) tc::mma_bf16(d + kNC, ad, bd, ID2, 1u);
        else tc::mma_bf16(d + 2 * kNC, ad, bd, ID1, 1u);
      }
  } else {
    constexpr uint32_t ID2 = tc::idesc_tf32(128, 2 * kNC), ID1 = tc::idesc_tf32(128, kNC);
    const int kt = u >> 1, sp = u & 1;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks)
#pragma unroll
      for (int tb = 0; tb < NT; ++tb) {
        if (tb < tb0 || tb >= tb1) continue;  // tables of the other MMA thread
        if (32 * kt + 8 * ks >= nk) continue;
        const uint32_t d = acc + (uint32_t)(tb * NACCS * kNC);
        const uint64_t ad = a0 + (uint64_t)((tb * 16384 + ks * 32) >> 4);
        const uint64_t bd = bd0 + (uint64_t)((tb * bstride_tb + kt * 2 * kNC * 128 + ks * 32) >> 4);
        if (sp == 0) tc::mma_tf32(d, ad, bd, ID2, (!first_chunk || kt || ks) ? 1u : 0u);
        else tc::mma_tf32(d + kNC, ad, bd, ID1, 1u);
      }
  }
}

// Pointer held by lane `src` (whole warp participates).
// Bytes of a 128-row table block that hold its first `rows` rows (8-row
// groups of 1 KB in the 128-byte-swizzled layout).  The rows past a block's
// colatitudes (synthesis) or degrees (analysis) are zero and are not loaded:
// the MMA reads whatever the ring slot held there into accumulator rows that
// the epilogue does not store.
__device__ __forceinline__ uint32_t table_rows_bytes(int rows) { return (uint32_t)((min(rows, 128) + 7) >> 3) << 10; }

template <typename P>
__device__ __forceinline__ P* shfl_ptr(P* p, int src) {
  const unsigned long long v = (unsigned long long)p;
  const unsigned lo = __shfl_sync(0xffffffffu, (unsigned)v, src);
  const unsigned hi = __shfl_sync(0xffffffffu, (unsigned)(v >> 32), src);
  return (P*)(((unsigned long long)hi << 32) | lo);
}

// Accumulators of one table summed smallest first, (C2 + C1) + C0 (bf16) or
// C1 + C0 (tf32), for the 32 columns at TMEM address `col` (this warp's lane
// quadrant).
template <bool TF32>
__device__ __forceinline__ void drain_sum(uint32_t col, float (&v)[32]) {
  uint32_t a[32], b[32];
  if (!TF32) {
    tc::tmem_ld32_nw(col + 2 * kNC, a);
    tc::tmem_ld32_nw(col + kNC, b);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(a[i]) + __uint_as_float(b[i]);
    tc::tmem_ld32_nw(col, a);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] += __uint_as_float(a[i]);
  } else {
    tc::tmem_ld32_nw(col + kNC, b);
    tc::tmem_ld32_nw(col, a);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(b[i]) + __uint_as_float(a[i]);
  }
}

// ------------------------------------------------------------------ packing
// One data tile per CTA (grid: column tile, m, tile of that m), built in
// shared memory and written with one bulk copy.
// Synthesis data images: [pc = bpc0[m] + p*nch + c][ct] tiles of 3 splits.
// One CTA builds both parity tiles of chunk c from 128 consecutive degrees.
using TcInv = LegInst<InvSet>;
using TcFwd = LegInst<FwdSet>;

template <bool VEC, bool TF32, bool MULTI>
__global__ void __launch_bounds__(kPackThreads, 4) pack_inv_kernel(const __grid_constant__ TcInv one,
                                                                  const TcInv* __restrict__ many,
                                                                  const __grid_constant__ InstIndex X) {
  constexpr int NC = kNC;
  constexpr uint32_t BSZ = Form<TF32>::OPSZ;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* B = align1k(smem_raw);
  int ct, mc, c;
  const TcInv& I = block_inst<MULTI>(one, many, X, ct, mc, c);
  const ShtGeom& g = I.g;
  const InvSet& s = I.s;
  const TcTables& t = I.t;
  unsigned char* __restrict__ bimg = I.bimg;
  const int nct = I.nct;
  const int m = mc * g.minc;
  const int nch = tc_nch(g.l_max - m + 1);
  if (c >= nch) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  inv_build_pair<VEC, NC, 1, TF32>(g, s, B, ct, ncplx, m, g.lmoff[mc], c, warp, kPackThreads / 32, lane);
  tc::fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    const long long pc = t.bpc0[mc] + c;  // parity 0; parity 1 is nch further
    tc::bulk_s2g(bimg + (pc * nct + ct) * (long long)BSZ, B, BSZ);
    tc::bulk_s2g(bimg + ((pc + nch) * nct + ct) * (long long)BSZ, B + BSZ, BSZ);
    tc::bulk_commit();
    tc::bulk_wait<0>();
  }
}

// Analysis data images: [m][c][ct] pairs (ES tile, EA tile) of 3 splits each,
// both built by one CTA from the (ES, EA) entries of 64 colatitudes.
template <bool VEC, bool TF32, bool MULTI>
__global__ void __launch_bounds__(kPackThreads, 4) pack_fwd_kernel(const __grid_constant__ TcFwd one,
                                                                  const TcFwd* __restrict__ many,
                                                                  const __grid_constant__ InstIndex X) {
  constexpr int NC = kNC;
  constexpr uint32_t PSZ = 2u * Form<TF32>::OPSZ;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* B = align1k(smem_raw);
  int ct, mc, c;
  const TcFwd& I = block_inst<MULTI>(one, many, X, ct, mc, c);
  const ShtGeom& g = I.g;
  const FwdSet& s = I.s;
  const TcTables& t = I.t;
  unsigned char* __restrict__ bimg = I.bimg;
  const int nct = I.nct;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  fwd_build_tile<VEC, NC, 2, true, TF32>(g, s, B, ct, ncplx, mc, 0, c, warp, kPackThreads / 32, lane);
  tc::fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::bulk_s2g(bimg + (((long long)mc * t.ncj + c) * nct + ct) * (long long)PSZ, B, PSZ);
    tc::bulk_commit();
    tc::bulk_wait<0>();
  }
}

// ------------------------------------------------------------ synthesis
struct InvTile {
  int mc, p, tt, ct, nch, nchp, nlp;
  __device__ void decode(const ShtGeom& g, const TcTables& t, int nct, int ix) {
    int rest;
    if (t.order == 0) {  // column tile fastest: consecutive tiles read the same table blocks
      ct = ix % nct;
      rest = ix / nct;
      tt = rest % t.ntt;
      rest /= t.ntt;
    } else {             // theta tile fastest: consecutive tiles read the same data tiles
      tt = ix % t.ntt;
      rest = ix / t.ntt;
      ct = rest % nct;
      rest /= nct;
    }
    p = rest & 1;
    mc = rest >> 1;
    const int n_l = g.l_max - mc * g.minc + 1;
    nch = tc_nch(n_l);
    nlp = (n_l + 1 - p) / 2;
    nchp = (nlp + 63) / 64;
  }
};

template <bool VEC, bool TF32, bool MULTI>
__global__ void __launch_bounds__(kThreads + Occ<VEC, TF32>::XTRA, Occ<VEC, TF32>::CPS)
    inv_leg_tcp(const __grid_constant__ TcInv one, const TcInv* __restrict__ many, const __grid_constant__ InstIndex X,
                int ntiles) {
  typedef Form<TF32> F;
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NC = kNC;
  constexpr int NA = Rings<VEC, true, TF32>::NA;
  constexpr int NB = Rings<VEC, true, TF32>::NB;
  constexpr uint32_t ACC = NT * F::NACCS * NC;  // one accumulator set
  constexpr int NACC = 2 * ACC <= Occ<VEC, TF32>::TCOLS ? 2 : 1;  // sets in the CTA's TMEM columns
  constexpr int BSZ = F::OPSZ;
  constexpr int ASZ = NT * 16384;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t a_full[NA], a_empty[NA], b_full[NB], b_empty[NB], acc_full[NACC], acc_empty[NACC], fin;
  __shared__ uint64_t tr_full[kNTR], tr_empty[kNTR];
  __shared__ int tr_idx[kNTR];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  unsigned char* base = align1k(smem_raw);
  unsigned char* sA = base;
  unsigned char* sB = sA + NA * ASZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    constexpr int NI = Occ<VEC, TF32>::NISS;
    for (int i = 0; i < NA; ++i) { tc::mbar_init(&a_full[i], 1); tc::mbar_init(&a_empty[i], NI); }
    for (int i = 0; i < NB; ++i) { tc::mbar_init(&b_full[i], 1); tc::mbar_init(&b_empty[i], NI); }
    for (int i = 0; i < NACC; ++i) { tc::mbar_init(&acc_full[i], NI); tc::mbar_init(&acc_empty[i], kEpiThreads); }
    tc::mbar_init(&fin, NI);
    for (int i = 0; i < kNTR; ++i) { tc::mbar_init(&tr_full[i], 1); tc::mbar_init(&tr_empty[i], NI + kEpiThreads); }
    s_fail = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, Occ<VEC, TF32>::TCOLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const TileRing R{tr_idx, tr_full, tr_empty};
  bool ok = true;
  InvTile T;

  if (warp == 0) {
    if (lane == 0) {  // ---------------------------------------- loader
      uint32_t a_use = 0, b_use = 0, tr = 0;
      int ix = blockIdx.x;
      while (ok) {
        if (!ring_push(R, tr, ix < ntiles ? ix : -1)) { ok = false; break; }
        if (ix >= ntiles) break;
        const int next = atomicAdd(one.t.tile_ctr, 1) + (int)gridDim.x;
        int lix = ix;
        const TcInv& I = tile_inst<MULTI>(one, many, X, lix);
        const ShtGeom& g = I.g;
        const TcTables& t = I.t;
        const int nct = I.nct;
        T.decode(g, t, nct, lix);
        ix = next;
        if (T.nlp == 0) continue;
        for (int c = 0; c < T.nchp && ok; ++c) {
          const uint32_t bslot = b_use % NB;
          if (!wait_empty(&b_empty[bslot], b_use, NB)) { ok = false; break; }
          tc::mbar_expect_tx(&b_full[bslot], BSZ);
          tc::bulk_g2s(sB + bslot * BSZ, I.bimg + ((t.bpc0[T.mc] + T.p * T.nch + c) * nct + T.ct) * (long long)BSZ,
                       BSZ, &b_full[bslot]);
          ++b_use;
          for (int u = 0; u < F::AUSES; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_empty(&a_empty[slot], a_use, NA)) { ok = false; break; }
            const uint32_t abytes = table_rows_bytes(g.nh - T.tt * 128);
            tc::mbar_expect_tx(&a_full[slot], NT * abytes);
            const int blk_u = TF32 ? 2 * (u & 1) + (u >> 1) : u;  // tf32 blocks: 2 * split + K tile
            for (int tb = 0; tb < NT; ++tb) {
              const long long blk =
                  t.inv_blk0[T.mc] + ((((long long)T.tt * 2 + tb) * 2 + T.p) * T.nch + c) * F::BPC + blk_u;
              tc::bulk_g2s(sA + slot * ASZ + tb * 16384, t.inv_img + blk * 16384, abytes, &a_full[slot]);
            }
          }
        }
      }
      drain_copies<NA>(a_full, a_use);
      drain_copies<NB>(b_full, b_use);
    }
  } else if (warp == 1 || (Occ<VEC, TF32>::NISS == 2 && warp == 2 + kEpiThreads / 32)) {
    if (lane == 0) {  // ---------------------------------------- MMA issuer(s)
      constexpr bool DUAL = Occ<VEC, TF32>::NISS == 2;
      const int tb0 = DUAL ? (warp == 1 ? 0 : 1) : 0, tb1 = DUAL ? tb0 + 1 : NT;
      uint32_t a_use = 0, b_use = 0, acc_use = 0, tr = 0;
      while (ok) {
        int ix;
        if (!ring_pop(R, tr, ix)) { ok = false; break; }
        if (ix < 0) break;
        const TcInv& I = tile_inst<MULTI>(one, many, X, ix);
        T.decode(I.g, I.t, I.nct, ix);
        if (T.nlp == 0) continue;
        const uint32_t abuf = acc_use % NACC;
        if (!wait_empty(&acc_empty[abuf], acc_use, NACC)) { ok = false; break; }
        tc::tc_fence_after();
        const uint32_t acc = tmem + abuf * ACC;
        for (int c = 0; c < T.nchp && ok; ++c, ++b_use) {
          const uint32_t bslot = b_use % NB;
          if (!wait_full(&b_full[bslot], b_use, NB)) { ok = false; break; }
          const int nk = min(64, T.nlp - 64 * c);  // K rows holding degrees of the order
          for (int u = 0; u < F::AUSES; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_full(&a_full[slot], a_use, NA)) { ok = false; break; }
            tc::tc_fence_after();
            issue_use<NT, TF32>(acc, sA + slot * ASZ, sB + bslot * BSZ, u, c == 0, 0, tb0, tb1, nk);
            tc::mma_commit(&a_empty[slot]);
          }
          tc::mma_commit(&b_empty[bslot]);
        }
        tc::mma_commit(&acc_full[abuf]);
        ++acc_use;
      }
      // every MMA issued above has finished before tensor memory is released
      tc::mma_commit(&fin);
      if (!tc::mbar_wait(&fin, 0)) ok = false;
    }
  } else if (warp < 2 + kEpiThreads / 32) {  // ---------------------- epilogue
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const int cc0 = half * (NC / 2);  // this warp's 32 real columns
    const int jl = 32 * q4 + lane;
    const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
    uint32_t acc_use = 0, tr = 0;
    while (ok) {
      int ix;
      if (!ring_pop(R, tr, ix)) { ok = false; break; }
      if (ix < 0) break;
      const TcInv& I = tile_inst<MULTI>(one, many, X, ix);
      const ShtGeom& g = I.g;
      const InvSet& s = I.s;
      const TcTables& t = I.t;
      const int npair = s.nf * s.nlev;
      const int ncplx = npair * (VEC ? 2 : 1);
      const int NHP = t.ntt * 128;
      T.decode(g, t, I.nct, ix);
      const int jg = T.tt * 128 + jl;
      const bool row_ok = jg < g.nh;
      // output column bases, one per lane, broadcast by shuffles: scalar: lane q <
      // 16 holds column q's array; vector: lane q < 8 the v_theta array of pair
      // q, lane 8 + q its v_phi array (E at +0, F at +nh)
      float2* cb = nullptr;
      {
        const long long per_p = VEC ? 2LL * g.nh : (long long)g.nh;
        const long long moff = ((long long)T.mc * 2 + T.p) * per_p;
        if (!VEC && lane < 16) {
          const int cq = T.ct * (NC / 2) + cc0 / 2 + lane;
          if (cq < ncplx) {
            const int r = cq / s.nf, f = cq - r * s.nf;
            cb = (float2*)s.f[f].out0 + (long long)r * s.f[f].out_ld + moff;
          }
        } else if (VEC && lane < 16) {
          const int pr = T.ct * (NC / 4) + cc0 / 4 + (lane & 7);
          if (pr < npair) {
            const int r = pr / s.nf, f = pr - r * s.nf;
            cb = (float2*)(lane < 8 ? s.f[f].out0 : s.f[f].out1) + (long long)r * s.f[f].out_ld + moff;
          }
        }
      }
      if (T.nlp == 0) {  // odd parity of m = l_max: zeros
        for (int q = 0; q < 16; ++q) {
          float2* b = shfl_ptr(cb, q);
          if (b && row_ok) {
            b[jg] = make_float2(0.f, 0.f);
            if (VEC) b[g.nh + jg] = make_float2(0.f, 0.f);
          }
        }
        continue;
      }
      const uint32_t abuf = acc_use % NACC;
      if (!wait_full(&acc_full[abuf], acc_use, NACC)) { ok = false; break; }
      tc::tc_fence_after();
      const uint32_t acc = tmem + abuf * ACC + lane_off + cc0;
      float P[32], D[32];
      drain_sum<TF32>(acc, P);
      if (VEC) drain_sum<TF32>(acc + F::NACCS * NC, D);
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_empty[abuf]);  // tensor memory free for the next tile
      ++acc_use;
      const float sP = row_ok ? t.inv_scale[(size_t)T.mc * NHP + jg] : 0.f;
#pragma unroll
      for (int i = 0; i < 32; ++i) P[i] *= sP;
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          float2* b = shfl_ptr(cb, q);
          if (b && row_ok) b[jg] = make_float2(P[2 * q], P[2 * q + 1]);
        }
      } else {
        const float sdP = row_ok ? t.inv_scale[((size_t)g.n_m + T.mc) * NHP + jg] : 0.f;
        const float dm = (float)(T.mc * g.minc);
#pragma unroll
        for (int i = 0; i < 32; ++i) D[i] *= sdP;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float2* bt = shfl_ptr(cb, q);
          float2* bp = shfl_ptr(cb, 8 + q);
          // C = sum S P, B = sum T P; A = sum S dP, D = sum T dP
          const float Cr = P[4 * q], Ci = P[4 * q + 1], Br = P[4 * q + 2], Bi = P[4 * q + 3];
          const float Ar = D[4 * q], Ai = D[4 * q + 1], Dr = D[4 * q + 2], Di = D[4 * q + 3];
          // v_theta: U = i m B, W = A;   v_phi: U = i m C, W = -D
          const float2 Ut = make_float2(-dm * Bi, dm * Br), Wt = make_float2(Ar, Ai);
          const float2 Up = make_float2(-dm * Ci, dm * Cr), Wp = make_float2(-Dr, -Di);
          if (bt && row_ok) {
            bt[jg] = make_float2(Ut.x + Wt.x, Ut.y + Wt.y);
            bt[g.nh + jg] = make_float2(Ut.x - Wt.x, Ut.y - Wt.y);
            bp[jg] = make_float2(Up.x + Wp.x, Up.y + Wp.y);
            bp[g.nh + jg] = make_float2(Up.x - Wp.x, Up.y - Wp.y);
          }
        }
      }
    }
  }
  if (!ok) atomicExch(&s_fail, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_fail && one.t.err) atomicExch(one.t.err, 1);
  if (warp == 0) tc::tmem_dealloc(tmem, Occ<VEC, TF32>::TCOLS);
}

// ------------------------------------------------------------ analysis
struct FwdTile {
  int mc, p, lt, ct, nlp;
  __device__ void decode(const ShtGeom& g, const TcTables& t, int nct, int ix) {
    int rest;
    if (t.order == 0) {  // column tile fastest: consecutive tiles read the same table blocks
      ct = ix % nct;
      rest = ix / nct;
      lt = rest % t.nlt;
      rest /= t.nlt;
    } else {             // degree tile fastest: consecutive tiles read the same data tiles
      lt = ix % t.nlt;
      rest = ix / t.nlt;
      ct = rest % nct;
      rest /= nct;
    }
    p = rest & 1;
    mc = rest >> 1;
    const int n_l = g.l_max - mc * g.minc + 1;
    nlp = (n_l + 1 - p) / 2;
  }
};

template <bool VEC, bool TF32, bool MULTI>
__global__ void __launch_bounds__(kThreads + Occ<VEC, TF32>::XTRA, Occ<VEC, TF32>::CPS)
    fwd_leg_tcp(const __grid_constant__ TcFwd one, const TcFwd* __restrict__ many, const __grid_constant__ InstIndex X,
                int ntiles) {
  typedef Form<TF32> F;
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NC = kNC;
  constexpr int NA = Rings<VEC, false, TF32>::NA;
  constexpr int NB = Rings<VEC, false, TF32>::NB;
  constexpr uint32_t ACC = NT * F::NACCS * NC;
  constexpr int NACC = 2 * ACC <= Occ<VEC, TF32>::TCOLS ? 2 : 1;
  constexpr int TS = F::OPSZ;       // one data operand
  constexpr int ASZ = NT * 16384;
  constexpr int BSZ = NT * TS;      // mine (and other)
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t a_full[NA], a_empty[NA], b_full[NB], b_empty[NB], acc_full[NACC], acc_empty[NACC], fin;
  __shared__ uint64_t tr_full[kNTR], tr_empty[kNTR];
  __shared__ int tr_idx[kNTR];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  unsigned char* base = align1k(smem_raw);
  unsigned char* sA = base;
  unsigned char* sB = sA + NA * ASZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    constexpr int NI = Occ<VEC, TF32>::NISS;
    for (int i = 0; i < NA; ++i) { tc::mbar_init(&a_full[i], 1); tc::mbar_init(&a_empty[i], NI); }
    for (int i = 0; i < NB; ++i) { tc::mbar_init(&b_full[i], 1); tc::mbar_init(&b_empty[i], NI); }
    for (int i = 0; i < NACC; ++i) { tc::mbar_init(&acc_full[i], NI); tc::mbar_init(&acc_empty[i], kEpiThreads); }
    tc::mbar_init(&fin, NI);
    for (int i = 0; i < kNTR; ++i) { tc::mbar_init(&tr_full[i], 1); tc::mbar_init(&tr_empty[i], NI + kEpiThreads); }
    s_fail = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, Occ<VEC, TF32>::TCOLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const TileRing R{tr_idx, tr_full, tr_empty};
  bool ok = true;
  FwdTile T;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t a_use = 0, b_use = 0, tr = 0;
      int ix = blockIdx.x;
      while (ok) {
        if (!ring_push(R, tr, ix < ntiles ? ix : -1)) { ok = false; break; }
        if (ix >= ntiles) break;
        const int next = atomicAdd(one.t.tile_ctr, 1) + (int)gridDim.x;
        int lix = ix;
        const TcFwd& I = tile_inst<MULTI>(one, many, X, lix);
        const TcTables& t = I.t;
        const int nct = I.nct;
        T.decode(I.g, t, nct, lix);
        ix = next;
        if (T.lt * 128 >= T.nlp) continue;
        for (int c = 0; c < t.ncj && ok; ++c) {
          const uint32_t bslot = b_use % NB;
          if (!wait_empty(&b_empty[bslot], b_use, NB)) { ok = false; break; }
          tc::mbar_expect_tx(&b_full[bslot], BSZ);
          const unsigned char* img = I.bimg + (((long long)T.mc * t.ncj + c) * nct + T.ct) * (2LL * TS);
          tc::bulk_g2s(sB + bslot * BSZ, img + T.p * TS, TS, &b_full[bslot]);                    // mine
          if (VEC) tc::bulk_g2s(sB + bslot * BSZ + TS, img + (1 - T.p) * TS, TS, &b_full[bslot]);  // other
          ++b_use;
          for (int u = 0; u < F::AUSES; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_empty(&a_empty[slot], a_use, NA)) { ok = false; break; }
            const uint32_t abytes = table_rows_bytes(T.nlp - T.lt * 128);
            tc::mbar_expect_tx(&a_full[slot], NT * abytes);
            const int blk_u = TF32 ? 2 * (u & 1) + (u >> 1) : u;
            for (int tb = 0; tb < NT; ++tb) {
              const long long blk =
                  t.fwd_blk0[T.mc] + ((((long long)T.p * t.nlt + T.lt) * 2 + tb) * t.ncj + c) * F::BPC + blk_u;
              tc::bulk_g2s(sA + slot * ASZ + tb * 16384, t.fwd_img + blk * 16384, abytes, &a_full[slot]);
            }
          }
        }
      }
      drain_copies<NA>(a_full, a_use);
      drain_copies<NB>(b_full, b_use);
    }
  } else if (warp == 1 || (Occ<VEC, TF32>::NISS == 2 && warp == 2 + kEpiThreads / 32)) {
    if (lane == 0) {  // MMA issuer(s)
      constexpr bool DUAL = Occ<VEC, TF32>::NISS == 2;
      const int tb0 = DUAL ? (warp == 1 ? 0 : 1) : 0, tb1 = DUAL ? tb0 + 1 : NT;
      uint32_t a_use = 0, b_use = 0, acc_use = 0, tr = 0;
      while (ok) {
        int ix;
        if (!ring_pop(R, tr, ix)) { ok = false; break; }
        if (ix < 0) break;
        const TcFwd& I = tile_inst<MULTI>(one, many, X, ix);
        T.decode(I.g, I.t, I.nct, ix);
        if (T.lt * 128 >= T.nlp) continue;
        const uint32_t abuf = acc_use % NACC;
        if (!wait_empty(&acc_empty[abuf], acc_use, NACC)) { ok = false; break; }
        tc::tc_fence_after();
        const uint32_t acc = tmem + abuf * ACC;
        for (int c = 0; c < I.t.ncj && ok; ++c, ++b_use) {
          const uint32_t bslot = b_use % NB;
          if (!wait_full(&b_full[bslot], b_use, NB)) { ok = false; break; }
          for (int u = 0; u < F::AUSES; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_full(&a_full[slot], a_use, NA)) { ok = false; break; }
            tc::tc_fence_after();
            issue_use<NT, TF32>(acc, sA + slot * ASZ, sB + bslot * BSZ, u, c == 0, TS, tb0, tb1);
            tc::mma_commit(&a_empty[slot]);
          }
          tc::mma_commit(&b_empty[bslot]);
        }
        tc::mma_commit(&acc_full[abuf]);
        ++acc_use;
      }
      tc::mma_commit(&fin);
      if (!tc::mbar_wait(&fin, 0)) ok = false;
    }
  } else if (warp < 2 + kEpiThreads / 32) {  // epilogue
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const int cc0 = half * (NC / 2);
    const int lr = 32 * q4 + lane;
    const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
    uint32_t acc_use = 0, tr = 0;
    while (ok) {
      int ix;
      if (!ring_pop(R, tr, ix)) { ok = false; break; }
      if (ix < 0) break;
      const TcFwd& I = tile_inst<MULTI>(one, many, X, ix);
      const ShtGeom& g = I.g;
      const FwdSet& s = I.s;
      const TcTables& t = I.t;
      const int npair = s.nf * s.nlev;
      const int ncplx = npair * (VEC ? 2 : 1);
      T.decode(g, t, I.nct, ix);
      if (T.lt * 128 >= T.nlp) continue;
      const uint32_t abuf = acc_use % NACC;
      if (!wait_full(&acc_full[abuf], acc_use, NACC)) { ok = false; break; }
      tc::tc_fence_after();
      const uint32_t acc = tmem + abuf * ACC + lane_off + cc0;
      float D0[32], D1[32];
      drain_sum<TF32>(acc, D0);
      if (VEC) drain_sum<TF32>(acc + F::NACCS * NC, D1);
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_empty[abuf]);
      ++acc_use;
      const int m = T.mc * g.minc;
      const int lp = T.lt * 128 + lr;
      const int l = m + T.p + 2 * lp;
      const bool valid = lp < T.nlp;
      const int lm = g.lmoff[T.mc] + l - m;
      // per-column output bases and cut-offs, one per lane, broadcast by shuffles:
      // scalar: lane q < 16 holds column q; vector: lane q < 8 pair q's S array,
      // lane 8 + q its T array
      double2* cb = nullptr;
      int clc = -1;
      if (lane < 16) {
        const int q = VEC ? (lane & 7) : lane;
        const int cq = VEC ? T.ct * (NC / 4) + cc0 / 4 + q : T.ct * (NC / 2) + cc0 / 2 + q;
        if (cq < (VEC ? npair : ncplx)) {
          const int r = cq / s.nf, f = cq - r * s.nf;
          cb = (VEC && lane >= 8 ? s.f[f].out1 : s.f[f].out0) + (long long)r * s.f[f].out_ld;
          clc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
        }
      }
      const float sP = valid ? t.fwd_scale[lm] : 0.f;
#pragma unroll
      for (int i = 0; i < 32; ++i) D0[i] *= sP;
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          double2* b = shfl_ptr(cb, q);
          const int lc = __shfl_sync(0xffffffffu, clc, q);
          if (b && valid)
            b[lm] = (l <= lc) ? make_double2(f2d_int(D0[2 * q]), f2d_int(D0[2 * q + 1])) : make_double2(0.0, 0.0);
        }
      } else {
        const float sdP = valid ? t.fwd_scale[(size_t)g.lm_max + lm] : 0.f;
        const float dm = (float)m;
        const float inv_ll = l > 0 ? 1.0f / (float)(l * (l + 1)) : 1.0f;
#pragma unroll
        for (int i = 0; i < 32; ++i) D1[i] *= sdP;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          double2* bs = shfl_ptr(cb, q);
          double2* bt = shfl_ptr(cb, 8 + q);
          const int lc = __shfl_sync(0xffffffffu, clc, q);
          // A = sum F1_mine P, D = sum F2_mine P, C = sum F1_other dP, B = sum F2_other dP
          const float Ar = D0[4 * q], Ai = D0[4 * q + 1], Dr = D0[4 * q + 2], Di = D0[4 * q + 3];
          const float Cr = D1[4 * q], Ci = D1[4 * q + 1], Br = D1[4 * q + 2], Bi = D1[4 * q + 3];
          double2 Sv = make_double2(f2d_int((dm * Ai + Br) * inv_ll), f2d_int((-dm * Ar + Bi) * inv_ll));
          double2 Tv = make_double2(f2d_int((-Cr + dm * Di) * inv_ll), f2d_int((-Ci - dm * Dr) * inv_ll));
          if (l > lc) { Sv = make_double2(0.0, 0.0); Tv = Sv; }
          if (bs && valid) {
            bs[lm] = Sv;
            bt[lm] = Tv;
          }
        }
      }
    }
  }
  if (!ok) atomicExch(&s_fail, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_fail && one.t.err) atomicExch(one.t.err, 1);
  if (warp == 0) tc::tmem_dealloc(tmem, Occ<VEC, TF32>::TCOLS);
}

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

int tcp_nct(int ncplx) { return (ncplx + kNC / 2 - 1) / (kNC / 2); }

template <bool VEC, bool TF32, bool MULTI>
cudaError_t launch_inv_p(const TcInv& one, const TcInv* many, const InstIndex& X, long long nblocks, long long ntiles,
                         cudaStream_t st) {
  constexpr int NT = VEC ? 2 : 1, NA = Rings<VEC, true, TF32>::NA, NB = Rings<VEC, true, TF32>::NB;
  constexpr size_t OPSZ = Form<TF32>::OPSZ;
  if (ntiles <= 0) return cudaSuccess;
  const size_t psmem = 1024 + 2 * OPSZ;
  CUDA_TRY(cudaFuncSetAttribute(pack_inv_kernel<VEC, TF32, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)psmem));
  const dim3 pgrid = MULTI ? dim3((unsigned)nblocks) : dim3(one.nct, one.g.n_m, tc_nch(one.g.l_max + 1));
  pack_inv_kernel<VEC, TF32, MULTI><<<pgrid, kPackThreads, psmem, st>>>(one, many, X);
  CUDA_TRY(cudaGetLastError());
  const size_t smem = 1024 + (size_t)NA * NT * 16384 + (size_t)NB * OPSZ;
  CUDA_TRY(cudaFuncSetAttribute(inv_leg_tcp<VEC, TF32, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::min<long long>(ntiles, (long long)num_sms() * Occ<VEC, TF32>::CPS);
  CUDA_TRY(cudaMemsetAsync(one.t.tile_ctr, 0, sizeof(int), st));
  inv_leg_tcp<VEC, TF32, MULTI><<<grid, kThreads + Occ<VEC, TF32>::XTRA, smem, st>>>(one, many, X, (int)ntiles);
  return cudaGetLastError();
}

template <bool VEC, bool TF32, bool MULTI>
cudaError_t launch_fwd_p(const TcFwd& one, const TcFwd* many, const InstIndex& X, long long nblocks, long long ntiles,
                         cudaStream_t st) {
  constexpr int NT = VEC ? 2 : 1, NA = Rings<VEC, false, TF32>::NA, NB = Rings<VEC, false, TF32>::NB;
  constexpr size_t OPSZ = Form<TF32>::OPSZ;
  if (ntiles <= 0) return cudaSuccess;
  const size_t psmem = 1024 + 2 * OPSZ;
  CUDA_TRY(cudaFuncSetAttribute(pack_fwd_kernel<VEC, TF32, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)psmem));
  const dim3 pgrid = MULTI ? dim3((unsigned)nblocks) : dim3(one.nct, one.g.n_m, one.t.ncj);
  pack_fwd_kernel<VEC, TF32, MULTI><<<pgrid, kPackThreads, psmem, st>>>(one, many, X);
  CUDA_TRY(cudaGetLastError());
  const size_t smem = 1024 + (size_t)NA * NT * 16384 + (size_t)NB * NT * OPSZ;
  CUDA_TRY(cudaFuncSetAttribute(fwd_leg_tcp<VEC, TF32, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::min<long long>(ntiles, (long long)num_sms() * Occ<VEC, TF32>::CPS);
  CUDA_TRY(cudaMemsetAsync(one.t.tile_ctr, 0, sizeof(int), st));
  fwd_leg_tcp<VEC, TF32, MULTI><<<grid, kThreads + Occ<VEC, TF32>::XTRA, smem, st>>>(one, many, X, (int)ntiles);
  return cudaGetLastError();
}

}  // namespace

size_t tcp_data_bytes(const ShtGeom& g, const TcTables& t, int ncplx, bool vec, bool inverse, bool tf32) {
  const int NC = kNC;
  (void)vec;
  const long long nct = (ncplx + NC / 2 - 1) / (NC / 2);
  const long long tile = tf32 ? (long long)Form<true>::OPSZ : (long long)Form<false>::OPSZ;
  if (inverse) return (size_t)(t.npc * nct * tile);
  return (size_t)((long long)g.n_m * t.ncj * nct * 2 * tile);
}

// tiles of the persistent kernels and blocks of the pack kernels of every
// instance (nct, tile0, blk0; g, s, t and bimg set by the caller)
template <class Set>
void tcp_layout_insts(LegInst<Set>* inst, int n, bool vec, long long* nblocks, long long* ntiles) {
  constexpr bool INV = std::is_same<Set, InvSet>::value;
  long long nb = 0, nt = 0;
  for (int i = 0; i < n; ++i) {
    LegInst<Set>& I = inst[i];
    const int ncplx = I.s.nf * I.s.nlev * (vec ? 2 : 1);
    I.nct = tcp_nct(ncplx > 0 ? ncplx : 0);
    I.cexp = nullptr;
    I.blk0 = (int)nb;
    I.tile0 = (int)nt;
    I.pad_ = 0;
    nb += (long long)I.nct * I.g.n_m * (INV ? tc_nch(I.g.l_max + 1) : I.t.ncj);
    nt += (long long)I.nct * (INV ? I.t.ntt : I.t.nlt) * 2 * I.g.n_m;
  }
  *nblocks = nb;
  *ntiles = nt;
}
template void tcp_layout_insts<InvSet>(LegInst<InvSet>*, int, bool, long long*, long long*);
template void tcp_layout_insts<FwdSet>(LegInst<FwdSet>*, int, bool, long long*, long long*);

cudaError_t launch_inv_legendre_tcp(const ShtGeom& g, const InvSet& s, bool vec, bool tf32, const TcTables& t,
                                    unsigned char* bimg, cudaStream_t st) {
  std::vector<TcInv> one(1);
  one[0].g = g;
  one[0].s = s;
  one[0].t = t;
  one[0].bimg = bimg;
  long long nb = 0, nt = 0;
  tcp_layout_insts(one.data(), 1, vec, &nb, &nt);
  const InstIndex X{};
  const TcInv& o = one[0];
  if (tf32)
    return vec ? launch_inv_p<true, true, false>(o, nullptr, X, nb, nt, st)
               : launch_inv_p<false, true, false>(o, nullptr, X, nb, nt, st);
  return vec ? launch_inv_p<true, false, false>(o, nullptr, X, nb, nt, st)
             : launch_inv_p<false, false, false>(o, nullptr, X, nb, nt, st);
}

cudaError_t launch_fwd_legendre_tcp(const ShtGeom& g, const FwdSet& s, bool vec, bool tf32, const TcTables& t,
                                    unsigned char* bimg, cudaStream_t st) {
  std::vector<TcFwd> one(1);
  one[0].g = g;
  one[0].s = s;
  one[0].t = t;
  one[0].bimg = bimg;
  long long nb = 0, nt = 0;
  tcp_layout_insts(one.data(), 1, vec, &nb, &nt);
  const InstIndex X{};
  const TcFwd& o = one[0];
  if (tf32)
    return vec ? launch_fwd_p<true, true, false>(o, nullptr, X, nb, nt, st)
               : launch_fwd_p<false, true, false>(o, nullptr, X, nb, nt, st);
  return vec ? launch_fwd_p<true, false, false>(o, nullptr, X, nb, nt, st)
             : launch_fwd_p<false, false, false>(o, nullptr, X, nb, nt, st);
}

// several instances of the 3xBF16 form in one pack + one persistent launch
cudaError_t launch_inv_legendre_tcp_multi(const LegInst<InvSet>* inst, const LegInst<InvSet>* d_inst, int n,
                                          bool vec, long long nblocks, long long ntiles, cudaStream_t st) {
  if (n < 1 || n > kMaxGroupInst) return cudaErrorInvalidValue;
  const InstIndex X = inst_index(inst, n);
  return vec ? launch_inv_p<true, false, true>(inst[0], d_inst, X, nblocks, ntiles, st)
             : launch_inv_p<false, false, true>(inst[0], d_inst, X, nblocks, ntiles, st);
}

cudaError_t launch_fwd_legendre_tcp_multi(const LegInst<FwdSet>* inst, const LegInst<FwdSet>* d_inst, int n,
                                          bool vec, long long nblocks, long long ntiles, cudaStream_t st) {
  if (n < 1 || n > kMaxGroupInst) return cudaErrorInvalidValue;
  const InstIndex X = inst_index(inst, n);
  return vec ? launch_fwd_p<true, false, true>(inst[0], d_inst, X, nblocks, ntiles, st)
             : launch_fwd_p<false, false, true>(inst[0], d_inst, X, nblocks, ntiles, st);
}

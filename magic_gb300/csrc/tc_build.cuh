// Builds of the data operand of the tensor-core Legendre sums, shared by
// the one-tile-per-CTA and the persistent kernels.
#pragma once
#include "common.cuh"
#include "cplx.cuh"

// ---------------------------------------------------------------------------
// Warp-cooperative builds of a whole data tile (B operand, K = 64 per chunk,
// rows 2ql / 2ql+1 = real / imaginary part of complex column ql).  A warp
// takes columns ql0, ql0 + qstride, ... in batches of CB: all global loads of
// a batch are issued first (lane = k and k + 32; 16-byte loads, consecutive
// lanes on consecutive entries), then the values are split to 3xBF16 and
// written with 2-byte stores into the 128-byte-swizzled K-major tiles.
#include <cuda_bf16.h>
#include "tc_ptx.cuh"

__device__ __forceinline__ void store_split1(unsigned char* tile0, uint32_t off, float v, uint32_t tile_bytes) {
  __nv_bfloat16 h, md, lo;
  tc::split3(v, h, md, lo);
  *(__nv_bfloat16*)(tile0 + off) = h;
  *(__nv_bfloat16*)(tile0 + tile_bytes + off) = md;
  *(__nv_bfloat16*)(tile0 + 2 * tile_bytes + off) = lo;
}

// Data operand of one tile: TF32 = false: 3 bf16 splits, NC rows each (split
// s at s * NC * 128 bytes); true: 2 K tiles of 32, each [hi rows | lo rows]
// (2 * NC rows, 16 KB for NC = 64).
template <bool TF32, int NC>
struct DataTile {
  static constexpr uint32_t bytes = TF32 ? 2u * 2u * NC * 128u : 3u * NC * 128u;
  static __device__ __forceinline__ void store(unsigned char* tile, int row, int k, float v) {
    if (!TF32) {
      store_split1(tile, tc::sw128_offset(row, k), v, NC * 128);
    } else {
      float hi, lo;
      tc::split_tf32(v, hi, lo);
      unsigned char* t = tile + (k >> 5) * (2 * NC * 128);
      *(float*)(t + tc::sw128_offset32(row, k & 31)) = hi;
      *(float*)(t + tc::sw128_offset32(NC + row, k & 31)) = lo;
    }
  }
};

template <bool VEC, int NC, int CB>
__device__ __forceinline__ void inv_build_tile(const ShtGeom& g, const InvSet& s, unsigned char* B, int ct,
                                               int ncplx, int m, int lm0, int p, int c, int ql0, int qstride,
                                               int lane) {
  constexpr uint32_t BT = NC * 128;
  const int lb = p + 128 * c;  // l - m of k = 0
  const int lmx = g.l_max - m;
  for (int qb = ql0; qb < NC / 2; qb += CB * qstride) {
    double2 a[CB][2], b[CB][2];
    int opk[CB], lc[CB];
    float o2[CB];
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      const int q = ct * (NC / 2) + ql;
      opk[i] = OP_ZERO;
      lc[i] = -1;
      o2[i] = 0.f;
      if (ql < NC / 2 && q < ncplx) {
        const int pair = VEC ? (q >> 1) : q;
        const int r = pair / s.nf, f = pair - r * s.nf;
        const SpecOperand& op = (VEC && (q & 1)) ? s.f[f].x1 : s.f[f].x0;
        if (op.op != OP_ZERO && op.A != nullptr) {
          opk[i] = op.op;
          const double2* A = op.A + (long long)r * op.ld + lm0;  // indexed by l - m
#pragma unroll
          for (int h = 0; h < 2; ++h) a[i][h] = __ldg(A + min(lb + 2 * (lane + 32 * h), lmx));
          if (op.op == OP_CURLT && op.B != nullptr) {
            const double2* Bp = op.B + (long long)r * op.ld + lm0;
#pragma unroll
            for (int h = 0; h < 2; ++h) b[i][h] = __ldg(Bp + min(lb + 2 * (lane + 32 * h), lmx));
            o2[i] = d2f_int(s.or2 ? s.or2[r] : s.or2_0);
          } else if (op.op == OP_CURLT) {
            opk[i] = OP_ZERO;
          }
          lc[i] = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
        }
      }
    }
    const float dm = (float)m;
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      if (ql >= NC / 2) break;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = lane + 32 * h;
        const int l = m + lb + 2 * k;
        float ar = 0.f, ai = 0.f;
        if (opk[i] != OP_ZERO) {
          ar = d2f_int(a[i][h].x);
          ai = d2f_int(a[i][h].y);
          const float ll = (float)(l * (l + 1));
          if (opk[i] == OP_DLH) {
            ar *= ll;
            ai *= ll;
          } else if (opk[i] == OP_CURLT) {
            const float d = o2[i] * ll;
            ar = fmaf(d, ar, -d2f_int(b[i][h].x));
            ai = fmaf(d, ai, -d2f_int(b[i][h].y));
          } else if (opk[i] == OP_IM) {
            const float t0 = ar;
            ar = -dm * ai;
            ai = dm * t0;
          }
          if (l > lc[i]) { ar = 0.f; ai = 0.f; }
        }
        store_split1(B, tc::sw128_offset(2 * ql, k), ar, BT);
        store_split1(B, tc::sw128_offset(2 * ql + 1, k), ai, BT);
      }
    }
  }
}

// Analysis tile: "mine" at B, "other" at B + 3 tiles (written when BOTH).
template <bool VEC, int NC, int CB, bool BOTH = VEC, bool TF32 = false>
__device__ __forceinline__ void fwd_build_tile(const ShtGeom& g, const FwdSet& s, unsigned char* B, int ct,
                                               int ncplx, int mc, int mine, int c, int ql0, int qstride,
                                               int lane) {
  for (int qb = ql0; qb < NC / 2; qb += CB * qstride) {
    float4 v[CB][2];
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      const int q = ct * (NC / 2) + ql;
      v[i][0] = v[i][1] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ql < NC / 2 && q < ncplx) {
        const int pair = VEC ? (q >> 1) : q;
        const int r = pair / s.nf, f = pair - r * s.nf;
        const float4* src = (const float4*)((const float2*)((VEC && (q & 1)) ? s.f[f].in1 : s.f[f].in0) +
                                            (long long)r * s.f[f].in_ld + (long long)mc * g.nh * 2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int j = 64 * c + lane + 32 * h;
          v[i][h] = __ldg(src + min(j, g.nh - 1));  // (ES, EA) at colatitude j
        }
      }
    }
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      if (ql >= NC / 2) break;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = lane + 32 * h;
        float4 x = v[i][h];
        if (64 * c + k >= g.nh) x = make_float4(0.f, 0.f, 0.f, 0.f);
        const float mr = mine ? x.z : x.x, mi = mine ? x.w : x.y;
        typedef DataTile<TF32, NC> DT;
        DT::store(B, 2 * ql, k, mr);
        DT::store(B, 2 * ql + 1, k, mi);
        if (BOTH) {
          const float orr = mine ? x.x : x.z, oi = mine ? x.y : x.w;
          DT::store(B + DT::bytes, 2 * ql, k, orr);
          DT::store(B + DT::bytes, 2 * ql + 1, k, oi);
        }
      }
    }
  }
}

// Both parity tiles of one 128-degree chunk c (degrees l = m + 128c + i,
// i < 128): tile p (p = i & 1) at B + p * 3 * NC * 128, K index (i >> 1).
// Lane holds i = lane + 32h (h < 4): each load instruction reads 32
// consecutive spectral entries, and both parities of every fetched sector are
// used.  The FP64 -> FP32 conversions use the hardware instruction here: at
// the pack kernel's occupancy they measured faster than the integer form.
template <bool VEC, int NC, int CB, bool TF32 = false>
__device__ __forceinline__ void inv_build_pair(const ShtGeom& g, const InvSet& s, unsigned char* B, int ct,
                                               int ncplx, int m, int lm0, int c, int ql0, int qstride,
                                               int lane) {
  const int lmx = g.l_max - m;
  for (int qb = ql0; qb < NC / 2; qb += CB * qstride) {
    double2 a[CB][4], b[CB][4];
    int opk[CB], lc[CB];
    float o2[CB];
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      const int q = ct * (NC / 2) + ql;
      opk[i] = OP_ZERO;
      lc[i] = -1;
      o2[i] = 0.f;
      if (ql < NC / 2 && q < ncplx) {
        const int pair = VEC ? (q >> 1) : q;
        const int r = pair / s.nf, f = pair - r * s.nf;
        const SpecOperand& op = (VEC && (q & 1)) ? s.f[f].x1 : s.f[f].x0;
        if (op.op != OP_ZERO && op.A != nullptr) {
          opk[i] = op.op;
          const double2* A = op.A + (long long)r * op.ld + lm0;  // indexed by l - m
#pragma unroll
          for (int h = 0; h < 4; ++h) a[i][h] = __ldg(A + min(128 * c + lane + 32 * h, lmx));
          if (op.op == OP_CURLT && op.B != nullptr) {
            const double2* Bp = op.B + (long long)r * op.ld + lm0;
#pragma unroll
            for (int h = 0; h < 4; ++h) b[i][h] = __ldg(Bp + min(128 * c + lane + 32 * h, lmx));
            o2[i] = __double2float_rn(s.or2 ? s.or2[r] : s.or2_0);
          } else if (op.op == OP_CURLT) {
            opk[i] = OP_ZERO;
          }
          lc[i] = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
        }
      }
    }
    const float dm = (float)m;
    typedef DataTile<TF32, NC> DT;
    unsigned char* Bp = B + (lane & 1) * DT::bytes;  // this lane's parity tile
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      const int ql = qb + i * qstride;
      if (ql >= NC / 2) break;
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int k = (lane >> 1) + 16 * h;
        const int l = m + 128 * c + lane + 32 * h;
        float ar = 0.f, ai = 0.f;
        if (opk[i] != OP_ZERO) {
          ar = __double2float_rn(a[i][h].x);
          ai = __double2float_rn(a[i][h].y);
          const float ll = (float)(l * (l + 1));
          if (opk[i] == OP_DLH) {
            ar *= ll;
            ai *= ll;
          } else if (opk[i] == OP_CURLT) {
            const float d = o2[i] * ll;
            ar = fmaf(d, ar, -__double2float_rn(b[i][h].x));
            ai = fmaf(d, ai, -__double2float_rn(b[i][h].y));
          } else if (opk[i] == OP_IM) {
            const float t0 = ar;
            ar = -dm * ai;
            ai = dm * t0;
          }
          if (l > lc[i]) { ar = 0.f; ai = 0.f; }
        }
        DT::store(Bp, 2 * ql, k, ar);
        DT::store(Bp, 2 * ql + 1, k, ai);
      }
    }
  }
}

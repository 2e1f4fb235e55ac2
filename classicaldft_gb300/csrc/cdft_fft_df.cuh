// FP64 transforms in double-float (df64) arithmetic on the FP32 pipe (cdft_df64.cuh),
// for the compile-time plans (128- and 256-point axes): the first stage of a transform
// reads doubles and splits them, the stages between keep df64 values in the tile (16
// bytes, as a double2), the last stage joins them back into doubles; IN_D / OUT_D = false
// leave the values in df64 for a caller that keeps computing in df64. Used by the tile
// passes (cdft_kernels_tma.cuh) and the row passes (cdft_kernels.cuh) in FP64.
#pragma once
#include <cuda_runtime.h>
#include "cdft_df64.cuh"
#include "cdft_fft.cuh"

namespace cdft {

// FP64 transforms of the compile-time plans run in df64 (tile and row passes)
constexpr bool kDf64Transforms = true;

// The df64 transforms take their own radix order for power-of-two lengths: radix-4
// stages, with a final radix-8 when the exponent is odd (128 = 4 4 8, 256 = 4 4 4 4).
// A tile of 8 FP64 columns gives a radix-8 stage only half as many butterflies as
// threads; last, its twiddles are all 1, so the idle half waits for the cheapest stage.
// Its twiddle table (same entry layout) follows the FP64 table of the default order.
__host__ __device__ constexpr int fxd_radix(int n, int i) {
  int m = n;
  for (int st = 0; m > 1; ++st) {
    int a = 0;
    while ((1 << (a + 1)) <= m) ++a;
    const int f = a == 3 ? 8 : (a >= 2 ? 4 : 2);
    if (st == i) return f;
    m /= f;
  }
  return 0;
}
__host__ __device__ constexpr int fxd_len(int n, int i) {
  int len = n;
  for (int st = 0; st < i; ++st) len /= fxd_radix(n, st);
  return len;
}
__host__ __device__ constexpr int fxd_twoff(int n, int i) {
  int off = 0, len = n;
  for (int st = 0; st < i; ++st) {
    const int p = fxd_radix(n, st);
    off += len + p;
    len /= p;
  }
  return off;
}
__host__ __device__ constexpr int fxd_table_len(int n) {
  int st = 0;
  while (fxd_radix(n, st) != 0) ++st;
  return fxd_twoff(n, st);
}

// a df64 twiddle from the plan's table staged in shared memory
__device__ __forceinline__ dfc ld_twiddle(const float4* p) {
  const float4 v = *p;
  dfc r;
  r.x = dfs(v.x, v.y);
  r.y = dfs(v.z, v.w);
  return r;
}

// The P-point DFTs of a df64 butterfly, with the sums that skip renormalisation
// (dfl_add, dfl_mul, dfl_dot2 in cdft_df64.cuh): inputs normalised pairs, outputs not.
__device__ __forceinline__ dfc dfcl_add(dfc a, dfc b) {
  dfc r;
  r.x = dfl_add(a.x, b.x);
  r.y = dfl_add(a.y, b.y);
  return r;
}
__device__ __forceinline__ dfc dfcl_sub(dfc a, dfc b) {
  dfc r;
  r.x = dfl_add(a.x, -b.x);
  r.y = dfl_add(a.y, -b.y);
  return r;
}
// a w (DIR < 0, forward) or a conj(w) (DIR > 0, backward)
template <int DIR>
__device__ __forceinline__ dfc dfcl_mul_dir(dfc a, dfc w) {
  dfc r;
  if constexpr (DIR < 0) {
    r.x = dfl_dot2(a.x, w.x, -a.y, w.y);
    r.y = dfl_dot2(a.x, w.y, a.y, w.x);
  } else {
    r.x = dfl_dot2(a.x, w.x, a.y, w.y);
    r.y = dfl_dot2(a.y, w.x, -a.x, w.y);
  }
  return r;
}
template <int DIR>
__device__ __forceinline__ void dft4_dfl(dfc* a) {
  const dfc t0 = dfcl_add(a[0], a[2]), t1 = dfcl_sub(a[0], a[2]), t2 = dfcl_add(a[1], a[3]),
            t3 = cmul_mi<DIR>(dfcl_sub(a[1], a[3]));
  a[0] = dfcl_add(t0, t2);
  a[2] = dfcl_sub(t0, t2);
  a[1] = dfcl_add(t1, t3);
  a[3] = dfcl_sub(t1, t3);
}
template <int DIR>
__device__ __forceinline__ void dft8_dfl(dfc* a) {
  constexpr dfs r(0.70710678118654752440084436210484903928);
  dfc e[4] = {a[0], a[2], a[4], a[6]}, o[4] = {a[1], a[3], a[5], a[7]};
  dft4_dfl<DIR>(e);
  dft4_dfl<DIR>(o);
  // w8^k for k = 1, 2, 3 on the odd half
  const dfc o1 = o[1], o3 = o[3];
  if constexpr (DIR < 0) {
    o[1].x = dfl_mul(r, dfl_add(o1.x, o1.y));
    o[1].y = dfl_mul(r, dfl_add(o1.y, -o1.x));
    o[3].x = dfl_mul(r, dfl_add(o3.y, -o3.x));
    o[3].y = -dfl_mul(r, dfl_add(o3.x, o3.y));
  } else {
    o[1].x = dfl_mul(r, dfl_add(o1.x, -o1.y));
    o[1].y = dfl_mul(r, dfl_add(o1.x, o1.y));
    o[3].x = -dfl_mul(r, dfl_add(o3.x, o3.y));
    o[3].y = dfl_mul(r, dfl_add(o3.x, -o3.y));
  }
  o[2] = cmul_mi<DIR>(o[2]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    a[k] = dfcl_add(e[k], o[k]);
    a[k + 4] = dfcl_sub(e[k], o[k]);
  }
}

template <int DIR, int P, int TC, bool UNIT, bool IN_D, bool OUT_D>
__device__ __forceinline__ void tile_butterfly_df(const void* __restrict__ xv, void* __restrict__ yv, int c, int q, int k, int m, int s,
                                                  const float4* __restrict__ tw) {
  dfc a[P];
#pragma unroll
  for (int j = 0; j < P; ++j) {
    const int idx = (k + s * (q + m * j)) * TC + c;
    if constexpr (IN_D) a[j] = dfc_split(reinterpret_cast<const double2*>(xv)[idx]);
    else a[j] = reinterpret_cast<const dfc*>(xv)[idx];
  }
  if constexpr (P == 8) dft8_dfl<DIR>(a);
  else if constexpr (P == 4) dft4_dfl<DIR>(a);
  else {
    const dfc t = a[0];
    a[0] = dfcl_add(t, a[1]);
    a[1] = dfcl_sub(t, a[1]);
  }
  const float4* twq = tw + q * P;
#pragma unroll
  for (int t = 0; t < P; ++t) {
    dfc v = (UNIT || t == 0) ? a[t] : dfcl_mul_dir<DIR>(a[t], ld_twiddle(twq + t));
    const int idx = (k + s * (P * q + t)) * TC + c;
    if constexpr (OUT_D) {
      reinterpret_cast<double2*>(yv)[idx] = dfc_join(v);  // hi + lo rounded once, normalised or not
    } else {
      if constexpr (UNIT) {  // the last stage: what leaves the transform is renormalised
        v.x = df_renorm(v.x);
        v.y = df_renorm(v.y);
      }
      reinterpret_cast<dfc*>(yv)[idx] = v;
    }
  }
}

// (no unrolling of the item loop: a df64 butterfly is ~12x the instructions of an FP64
// one, and unrolled copies of every stage overflowed the instruction cache)
// ncols < TC: a partial tile (the last column tile of a half spectrum), whose first ncols
// columns alone are transformed, their butterflies packed onto the first threads so that
// the other warps skip the stage; the last stage writes zeros into the other columns.
template <int DIR, int TC, int PITCH, int NF, int ST, int NTH, bool IN_D, bool OUT_D>
__device__ __forceinline__ void fx_stage_df(const void* __restrict__ src, void* __restrict__ dst, const float4* __restrict__ tws,
                                            int ncols) {
  constexpr int p = fxd_radix(NF, ST), len = fxd_len(NF, ST), m = len / p, s = NF / len;
  constexpr bool first = IN_D && ST == 0, final_stage = fxd_radix(NF, ST + 1) == 0, last = OUT_D && final_stage;
  static_assert(p == 2 || p == 4 || p == 8, "df64 stages take radices 2, 4 and 8");
  const float4* tw = tws + fxd_twoff(NF, ST);
  const bool full = ncols >= TC;
  const int items = (full ? TC : ncols) * (NF / p);
#pragma unroll 1
  for (int w = threadIdx.x; w < items; w += NTH) {
    const int c = full ? w % TC : w % ncols, u = full ? w / TC : w / ncols;
    const int q = u / s, k = u % s;
    tile_butterfly_df<DIR, p, PITCH, m == 1, first, last>(src, dst, c, q, k, m, s, tw);
  }
  if (final_stage && !full) {
    const int dead = TC - ncols;
    for (int w = threadIdx.x; w < dead * NF; w += NTH) {
      const int idx = (w / dead) * PITCH + ncols + w % dead;
      if constexpr (OUT_D) reinterpret_cast<double2*>(dst)[idx] = make_double2(0.0, 0.0);
      else reinterpret_cast<dfc*>(dst)[idx] = dfc{dfs(0), dfs(0)};
    }
  }
}

template <int DIR, int TC, int PITCH, int NF, int NTH, bool IN_D, bool OUT_D, int ST = 0>
__device__ __forceinline__ double2* tile_fft_fixed_df_stages(double2* b0, double2* b1, const float4* __restrict__ tws, int ncols) {
  __syncthreads();
  if constexpr (fxd_radix(NF, ST) == 0) {
    return b0;
  } else {
    fx_stage_df<DIR, TC, PITCH, NF, ST, NTH, IN_D, OUT_D>(b0, b1, tws, ncols);
    return tile_fft_fixed_df_stages<DIR, TC, PITCH, NF, NTH, IN_D, OUT_D, ST + 1>(b1, b0, tws, ncols);
  }
}
// Each call stages the plan's df64 twiddles (fxd_table_len(NF) entries, 2.7 KB for 128
// points) in shared memory first: read by every butterfly, they made the texture path
// the bottleneck when fetched from global memory. The previous call ended on a barrier,
// so the copy cannot overwrite twiddles still in use. IN_D / OUT_D: the tile holds
// doubles on entry / exit (else df64 values, for a caller that keeps them).
template <int DIR, int TC, int PITCH, int NF, int NTH, bool IN_D = true, bool OUT_D = true>
__device__ __forceinline__ double2* tile_fft_fixed_df(double2* b0, double2* b1, const dfc* __restrict__ twdf, int ncols = TC) {
  constexpr int NT = fxd_table_len(NF);
  __shared__ float4 tws[NT];
  for (int i = threadIdx.x; i < NT; i += NTH) tws[i] = __ldg(reinterpret_cast<const float4*>(twdf) + i);
  return tile_fft_fixed_df_stages<DIR, TC, PITCH, NF, NTH, IN_D, OUT_D>(b0, b1, tws, ncols);
}


// The same transform on RB rows of length NF held line-contiguously (row r at r * LP),
// the layout of the row passes.
template <int DIR, int NF, int NTH, bool IN_D, bool OUT_D, int ST = 0>
__device__ __forceinline__ double2* rows_fft_df_stages(double2* b0, double2* b1, int L, int LP, const float4* __restrict__ tws) {
  __syncthreads();
  if constexpr (fxd_radix(NF, ST) == 0) {
    return b0;
  } else {
    constexpr int p = fxd_radix(NF, ST), len = fxd_len(NF, ST), m = len / p, s = NF / len, per_line = NF / p;
    constexpr bool first = IN_D && ST == 0, last = OUT_D && fxd_radix(NF, ST + 1) == 0;
    const float4* tw = tws + fxd_twoff(NF, ST);
#pragma unroll 1
    for (int w = threadIdx.x; w < L * per_line; w += NTH) {
      const int line = w / per_line, u = w - line * per_line;
      const int q = u / s, k = u % s;
      tile_butterfly_df<DIR, p, 1, m == 1, first, last>(b0 + (long)line * LP, b1 + (long)line * LP, 0, q, k, m, s, tw);
    }
    return rows_fft_df_stages<DIR, NF, NTH, IN_D, OUT_D, ST + 1>(b1, b0, L, LP, tws);
  }
}
template <int DIR, int NF, int NTH, bool IN_D = true, bool OUT_D = true>
__device__ __forceinline__ double2* rows_fft_df(double2* b0, double2* b1, int L, int LP, const dfc* __restrict__ twdf) {
  constexpr int NT = fxd_table_len(NF);
  __shared__ float4 tws[NT];
  for (int i = threadIdx.x; i < NT; i += NTH) tws[i] = __ldg(reinterpret_cast<const float4*>(twdf) + i);
  return rows_fft_df_stages<DIR, NF, NTH, IN_D, OUT_D>(b0, b1, L, LP, tws);
}

// offset of the df64 twiddles after the FP64 table of the default plan of length n
__host__ __device__ constexpr int df_table_offset(int n) {
  int st = 0;
  while (radix_at(n, st) != 0) ++st;
  return twoff_at(n, st);
}

// The row passes' transform: in df64 for FP64 with a compile-time plan, else block_fft_nf.
// IN_D / OUT_D as for tile_fft_fixed_df (df64 only).
template <int DIR, class T, int NF, bool IN_D = true, bool OUT_D = true>
__device__ __forceinline__ typename Cx<T>::type* rows_fft(typename Cx<T>::type* b0, typename Cx<T>::type* b1, int L, int LP, const FFTPlan& P,
                                                          const typename Cx<T>::type* __restrict__ table) {
  if constexpr (kDf64Transforms && NF > 0 && sizeof(T) == 8) {
    double2* r = rows_fft_df<DIR, NF, 256, IN_D, OUT_D>(b0, b1, L, LP, reinterpret_cast<const dfc*>(table + df_table_offset(NF)));
    __syncthreads();
    return r;
  } else {
    return block_fft_nf<DIR, T, NF>(b0, b1, L, LP, P, table);
  }
}

}  // namespace cdft

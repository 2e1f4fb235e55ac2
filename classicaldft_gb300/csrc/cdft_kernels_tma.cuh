// TMA-fed column passes (sm_103a). A tile is TC consecutive columns of the
// padded half spectrum by the n points of the transform axis, stored row-major
// [n][TC] in shared memory exactly as the tensor copy writes it. Threads map
// column-fastest onto the tile, so every FFT stage reads and writes shared
// memory without bank conflicts, and no padding is needed.
//
// Each kernel keeps two tiles in flight: while one is transformed, the tensor
// engine brings the next one in, with an mbarrier per stage buffer. Results
// leave through tensor stores from shared memory.
#pragma once
#include <type_traits>
#include "cdft_fft_df.cuh"
#include "cdft_kernels.cuh"
#include "cdft_tma.cuh"

namespace cdft {

// Radix-P butterfly on column c of a row-major tile with TC columns.
// TC here is the tile's row pitch in complex elements (>= the column count).
// UNIT: every stage twiddle is 1 (the last stage of a plan, m = 1, where q = 0):
// the products with them are skipped, which leaves every value's bits unchanged.
template <int DIR, class T, int P, int TC, bool UNIT = false>
__device__ __forceinline__ void tile_butterfly(const typename Cx<T>::type* __restrict__ x, typename Cx<T>::type* __restrict__ y, int c,
                                               int q, int k, int m, int s, const typename Cx<T>::type* __restrict__ tw,
                                               const typename Cx<T>::type* __restrict__ roots) {
  typedef typename Cx<T>::type C;
  C a[P];
#pragma unroll
  for (int j = 0; j < P; ++j) a[j] = x[(k + s * (q + m * j)) * TC + c];
  if (P == 8) {
    dft8<DIR, T>(a);
  } else if (P == 4) {
    dft4<DIR>(a);
  } else if (P == 2) {
    dft2<DIR>(a);
  } else {
    C w[P], b[P];
#pragma unroll
    for (int j = 0; j < P; ++j) w[j] = __ldg(reinterpret_cast<const C*>(roots + j));
#pragma unroll
    for (int t = 0; t < P; ++t) {
      C acc = a[0];
#pragma unroll
      for (int j = 1; j < P; ++j) acc = cadd(acc, cmul_dir<DIR>(a[j], w[(j * t) % P]));
      b[t] = acc;
    }
#pragma unroll
    for (int t = 0; t < P; ++t) a[t] = b[t];
  }
  const C* twq = tw + q * P;
  y[(k + s * (P * q)) * TC + c] = a[0];
#pragma unroll
  for (int t = 1; t < P; ++t) {
    if constexpr (UNIT) y[(k + s * (P * q + t)) * TC + c] = a[t];
    else y[(k + s * (P * q + t)) * TC + c] = cmul_dir<DIR>(a[t], __ldg(reinterpret_cast<const C*>(twq + t)));
  }
}

// Odd radices out of line: keeps their register arrays out of the kernels'
// register budget (the power-of-two lengths only inline radices 8, 4, 2).
template <int DIR, class T, int P, int TC>
__device__ __noinline__ void tile_butterfly_odd(const typename Cx<T>::type* __restrict__ x, typename Cx<T>::type* __restrict__ y, int c,
                                                int q, int k, int m, int s, const typename Cx<T>::type* __restrict__ tw,
                                                const typename Cx<T>::type* __restrict__ roots) {
  tile_butterfly<DIR, T, P, TC>(x, y, c, q, k, m, s, tw, roots);
}

template <int DIR, class T, int TC>
__device__ __noinline__ void tile_butterfly_generic(const typename Cx<T>::type* __restrict__ x, typename Cx<T>::type* __restrict__ y,
                                                    int c, int q, int k, int m, int s, int p, const typename Cx<T>::type* __restrict__ tw,
                                                    const typename Cx<T>::type* __restrict__ roots) {
  typedef typename Cx<T>::type C;
  C in[kMaxRadix];
  for (int j = 0; j < p; ++j) in[j] = x[(k + s * (q + m * j)) * TC + c];
  const C* twq = tw + q * p;
  for (int t = 0; t < p; ++t) {
    C acc = in[0];
    int idx = 0;
    for (int j = 1; j < p; ++j) {
      idx += t;
      if (idx >= p) idx -= p;
      acc = cadd(acc, cmul_dir<DIR>(in[j], roots[idx]));
    }
    y[(k + s * (p * q + t)) * TC + c] = (t == 0) ? acc : cmul_dir<DIR>(acc, twq[t]);
  }
}

// Transforms the TC columns of the tile in b0 (row pitch PITCH >= TC complex
// values; b1 is scratch); returns the buffer holding the result. Starts and
// ends with __syncthreads().
template <int DIR, class T, int TC, int PITCH = TC>
__device__ typename Cx<T>::type* tile_fft(typename Cx<T>::type* b0, typename Cx<T>::type* b1, const FFTPlan& P,
                                          const typename Cx<T>::type* __restrict__ table) {
  typedef typename Cx<T>::type C;
  C* src = b0;
  C* dst = b1;
  int len = P.n, s = 1;
  for (int st = 0; st < P.nst; ++st) {
    const int p = P.radix[st];
    const int m = len / p;
    const int items = TC * (P.n / p);
    const C* tw = table + P.tw_off[st];
    const C* rt = table + P.root_off[st];
    const int sh = ((s & (s - 1)) == 0) ? __ffs(s) - 1 : -1;  // stride as a shift when a power of two
    __syncthreads();
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
      const int c = w % TC, u = w / TC;
      int q, k;
      if (sh >= 0) {
        q = u >> sh;
        k = u & (s - 1);
      } else {
        q = u / s;
        k = u - q * s;
      }
      switch (p) {
        case 8: tile_butterfly<DIR, T, 8, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        case 4: tile_butterfly<DIR, T, 4, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        case 2: tile_butterfly<DIR, T, 2, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        case 3: tile_butterfly_odd<DIR, T, 3, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        case 5: tile_butterfly_odd<DIR, T, 5, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        case 7: tile_butterfly_odd<DIR, T, 7, PITCH>(src, dst, c, q, k, m, s, tw, rt); break;
        default: tile_butterfly_generic<DIR, T, PITCH>(src, dst, c, q, k, m, s, p, tw, rt); break;
      }
    }
    C* t = src;
    src = dst;
    dst = t;
    len = m;
    s *= p;
  }
  __syncthreads();
  return src;
}

// ---- fixed-length transforms: the plan of length NF (default radix order,
// largest radix first, as make_fft_table builds it) resolved at compile time,
// so every stride, trip count and twiddle offset is a constant.
__host__ __device__ constexpr int fx_radix(int n, int i) {
  int m = n;
  for (int st = 0; m > 1; ++st) {
    int f = 0;
    if (m % 8 == 0 && m != 16) f = 8;
    else if (m % 4 == 0) f = 4;
    else if (m % 2 == 0) f = 2;
    else {
      for (int q = 3; q <= m; q += 2)
        if (m % q == 0) { f = q; break; }
    }
    if (st == i) return f;
    m /= f;
  }
  return 0;
}
__host__ __device__ constexpr int fx_len(int n, int i) {
  int len = n;
  for (int st = 0; st < i; ++st) len /= fx_radix(n, st);
  return len;
}
// offset of stage i's twiddles in the table: each earlier stage holds len twiddles and p roots
__host__ __device__ constexpr int fx_twoff(int n, int i) {
  int off = 0, len = n;
  for (int st = 0; st < i; ++st) {
    const int p = fx_radix(n, st);
    off += len + p;
    len /= p;
  }
  return off;
}

template <int DIR, class T, int TC, int PITCH, int NF, int ST, int NTH>
__device__ __forceinline__ void fx_stage(const typename Cx<T>::type* __restrict__ src, typename Cx<T>::type* __restrict__ dst,
                                         const typename Cx<T>::type* __restrict__ table) {
  constexpr int p = fx_radix(NF, ST), len = fx_len(NF, ST), m = len / p, s = NF / len;
  constexpr int items = TC * (NF / p);
  const typename Cx<T>::type* tw = table + fx_twoff(NF, ST);
  const typename Cx<T>::type* rt = tw + len;
#pragma unroll 2
  for (int w = threadIdx.x; w < items; w += NTH) {
    const int c = w % TC, u = w / TC;
    const int q = u / s, k = u % s;
    if constexpr (p == 2 || p == 4 || p == 8) tile_butterfly<DIR, T, p, PITCH, m == 1>(src, dst, c, q, k, m, s, tw, rt);
    else if constexpr (p == 3 || p == 5 || p == 7) tile_butterfly_odd<DIR, T, p, PITCH>(src, dst, c, q, k, m, s, tw, rt);
    else tile_butterfly_generic<DIR, T, PITCH>(src, dst, c, q, k, m, s, p, tw, rt);
  }
}

template <int DIR, class T, int TC, int PITCH, int NF, int NTH, int ST = 0>
__device__ __forceinline__ typename Cx<T>::type* tile_fft_fixed(typename Cx<T>::type* b0, typename Cx<T>::type* b1,
                                                                const typename Cx<T>::type* __restrict__ table) {
  __syncthreads();
  if constexpr (fx_radix(NF, ST) == 0) {
    return b0;
  } else {
    fx_stage<DIR, T, TC, PITCH, NF, ST, NTH>(b0, b1, table);
    return tile_fft_fixed<DIR, T, TC, PITCH, NF, NTH, ST + 1>(b1, b0, table);
  }
}

// ---- FP64 transforms in df64 arithmetic: cdft_fft_df.cuh.
__host__ __device__ constexpr int fx_nstages(int n) {
  int st = 0;
  while (fx_radix(n, st) != 0) ++st;
  return st;
}
__host__ __device__ constexpr int fx_table_len(int n) { return fx_twoff(n, fx_nstages(n)); }

// The transform of a tile: the compile-time plan when NF > 0 (launched only
// when the runtime plan is that default plan of length NF), else the runtime plan.
template <int DIR, class T, int TC, int PITCH, int NF, int NTH = 256>
__device__ __forceinline__ typename Cx<T>::type* tfft(typename Cx<T>::type* b0, typename Cx<T>::type* b1, const FFTPlan& P,
                                                      const typename Cx<T>::type* __restrict__ table) {
  if constexpr (NF > 0 && kDf64Transforms && std::is_same<T, double>::value)
    return tile_fft_fixed_df<DIR, TC, PITCH, NF, NTH>(b0, b1, reinterpret_cast<const dfc*>(table + fx_table_len(NF)));
  else if constexpr (NF > 0) return tile_fft_fixed<DIR, T, TC, PITCH, NF, NTH>(b0, b1, table);
  else return tile_fft<DIR, T, TC, PITCH>(b0, b1, P, table);
}

// Tile geometry: TC complex columns make one 128-byte row.
template <class T> struct TileCols;
template <> struct TileCols<float> { static constexpr int value = 16; };
template <> struct TileCols<double> { static constexpr int value = 8; };
// the y pass's tiles: 16 columns in both precisions (256-byte FP64 rows), so that every
// stage of a df64 transform has a butterfly for each of the 256 threads (12-column FP64
// tiles, three blocks per SM instead of two, measured 9% slower)
template <class T> struct TileColsY { static constexpr int value = 16; };
// rows per group of the fused Phi kernel
template <class T> struct PhiRows;
template <> struct PhiRows<float> { static constexpr int value = 4; };
template <> struct PhiRows<double> { static constexpr int value = 2; };
// rows per group for a compile-time row length: half as many for 256-point rows
template <class T, int NF> struct PhiRowsFor {
  static constexpr int value = NF == 256 ? (PhiRows<T>::value > 1 ? PhiRows<T>::value / 2 : 1) : PhiRows<T>::value;
};
// 8-byte tensor elements per complex value (float2 = 1, double2 = 2)
template <class T> struct ElemsPerComplex;
template <> struct ElemsPerComplex<float> { static constexpr int value = 1; };
template <> struct ElemsPerComplex<double> { static constexpr int value = 2; };

// The x passes' transforms. In FP64 with a compile-time plan they run in df64 and may
// leave (OUT_D = false) or take (IN_D = false) df64 values, so that the products with
// the weights happen in df64 too and no join / split pair surrounds them; XReg is the
// type a thread holds such values in.
// ncols (df64 only): the tile's live columns, as for tile_fft_fixed_df.
template <int DIR, class T, int TC, int NF, bool IN_D, bool OUT_D>
__device__ __forceinline__ typename Cx<T>::type* xfft(typename Cx<T>::type* b0, typename Cx<T>::type* b1, const FFTPlan& P,
                                                      const typename Cx<T>::type* __restrict__ tw, int ncols = TC) {
  if constexpr (kDf64Transforms && std::is_same<T, double>::value && NF > 0)
    return tile_fft_fixed_df<DIR, TC, TC, NF, 256, IN_D, OUT_D>(b0, b1, reinterpret_cast<const dfc*>(tw + fx_table_len(NF)), ncols);
  else
    return tfft<DIR, T, TC, TC, NF>(b0, b1, P, tw);
}
template <class T, int NF> struct XReg {
  static constexpr bool df = kDf64Transforms && std::is_same<T, double>::value && NF > 0;
  typedef typename std::conditional<df, dfc, typename Cx<T>::type>::type C;  // a complex value
  typedef typename std::conditional<df, dfs, T>::type W;                      // a weight
  __device__ static W weight(T w) {
    if constexpr (df) return dfs_split((double)w);
    else return w;
  }
  // weight e of a staged tile: FP64 weights split here, or (DFS) weights stored as df64
  template <bool DFS>
  __device__ static W load_weight(const T* tile, int e) {
    if constexpr (df && DFS) return reinterpret_cast<const dfs*>(tile)[e];
    else return weight(tile[e]);
  }
  __device__ static C zero() {
    C z;
    if constexpr (df) z.x = z.y = dfs(0);
    else z.x = z.y = (T)0;
    return z;
  }
  __device__ static T re(const C& z) {
    if constexpr (df) return (T)dfs_join(z.x);
    else return z.x;
  }
  __device__ static T im(const C& z) {
    if constexpr (df) return (T)dfs_join(z.y);
    else return z.y;
  }
};

// ---------------------------------------------------------------- y pass ---
// Work item = (field f, plane x, column tile t): the tile [ny][TC] at kz0 = t*TC.
// Tensor map (4D, 8-byte elements): {pz*E, ny, nx, nfield}.
template <class T, int DIR, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256) k_cols_y_tma(const __grid_constant__ CUtensorMap map, Dims d, FFTPlan P,
                                                    const typename Cx<T>::type* __restrict__ tw, int nfield, unsigned* __restrict__ status) {
  typedef typename Cx<T>::type C;
  constexpr int TC = TileColsY<T>::value, E = ElemsPerComplex<T>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* sm = aligned_smem(smem_raw);
  const int n = P.n;
  const size_t tile_bytes = (size_t)n * TC * sizeof(C), tb = r128(tile_bytes);
  // buffers by address arithmetic (an array of pointers indexed by the stage would live in
  // local memory)
  auto stage = [&](int b) { return reinterpret_cast<C*>(sm + (size_t)b * tb); };
  C* work = reinterpret_cast<C*>(sm + 2 * tb);
  __shared__ __align__(8) uint64_t bar[2];
  const int ntile = (d.nzc + TC - 1) / TC;
  const long total = (long)nfield * d.nx * ntile;
  auto coords = [&](long item, int& kz0, int& x, int& f) {
    const int t = (int)(item % ntile);
    const long r = item / ntile;
    x = (int)(r % d.nx);
    f = (int)(r / d.nx);
    kz0 = t * TC;
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](long item, int b) {
    int kz0, x, f;
    coords(item, kz0, x, f);
    mbar_arrive_expect_tx(&bar[b], (unsigned)tile_bytes);
    tma_load_4d(stage(b), &map, kz0 * E, 0, x, f, &bar[b]);
  };
  if (threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b) {
      const long item = blockIdx.x + (long)b * gridDim.x;
      if (item < total) issue(item, b);
    }
  }
  bool ok = true;
  for (long k = 0;; ++k) {
    const long item = blockIdx.x + k * gridDim.x;
    if (item >= total) break;
    const int b = (int)(k & 1);
    ok = mbar_wait(&bar[b], (unsigned)((k >> 1) & 1), status);
    // the previous tile's store must have read its source (work, or its stage
    // buffer) before this tile's transform writes work
    if (threadIdx.x == 0) bulk_wait_read();
    if (!__syncthreads_and(ok)) break;
    int kz0, x, f;
    coords(item, kz0, x, f);
    // the last column tile holds nzc - kz0 live columns (one of 16 at 128 points)
    C* res = xfft<DIR, T, TC, NF, !DFS, !DFS>(stage(b), work, P, tw, min(TC, d.nzc - kz0));
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store_4d(&map, kz0 * E, 0, x, f, res);
      bulk_commit();
      const long next = item + 2L * gridDim.x;
      if (next < total) {
        if (res == stage(b)) bulk_wait_read();  // the store reads the buffer about to be refilled
        issue(next, b);
      }
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

// --------------------------------------------------------------- x passes ---
// Column tiles of the x pass: TC consecutive columns of the (ny*pz) column
// space, all nx rows. Maps (3D, rows = nx, third index = field):
//   complex fields {ncol*E, nx, nf} (8-byte elements); real weights {ncol, nx, nw}.

// C[a] = IFFT_x(FFT_x(A) . w_a) for a < M. The density spectrum lives in
// registers; weight tiles are double-buffered; results leave by tensor store.
template <class T, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256, 2) k_xconv_tma(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapW,
                                                   const __grid_constant__ CUtensorMap mapC, int M, FFTPlan px,
                                                   const typename Cx<T>::type* __restrict__ tw, unsigned* __restrict__ status) {
  typedef typename Cx<T>::type C;
  constexpr int TC = TileCols<T>::value, E = ElemsPerComplex<T>::value;
  constexpr int PER = TC;  // complex values a thread owns: n*TC/256 <= TC for n <= 256
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* sm = aligned_smem(smem_raw);
  const int n = px.n;
  const size_t tile_bytes = (size_t)n * TC * sizeof(C), wbytes = (size_t)n * TC * sizeof(T);
  const size_t tb = r128(tile_bytes), wb = r128(wbytes);
  C* X = reinterpret_cast<C*>(sm);
  C* Y = reinterpret_cast<C*>(sm + tb);
  auto Wst = [&](int b) { return reinterpret_cast<T*>(sm + 2 * tb + (size_t)b * wb); };  // not a pointer array (local memory)
  __shared__ __align__(8) uint64_t bar[3];  // 0, 1: weights; 2: density tile
  const int col0 = blockIdx.x * TC;
  const int nel = n * TC;
  if (threadIdx.x == 0) {
    for (int b = 0; b < 3; ++b) mbar_init(&bar[b], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar[2], (unsigned)tile_bytes);
    tma_load_3d(X, &mapA, col0 * E, 0, 0, &bar[2]);
    for (int b = 0; b < 2 && b < M; ++b) {
      mbar_arrive_expect_tx(&bar[b], (unsigned)wbytes);
      tma_load_3d(Wst(b), &mapW, col0, 0, b, &bar[b]);
    }
  }
  bool ok = mbar_wait(&bar[2], 0, status);
  if (!__syncthreads_and(ok)) {
    if (threadIdx.x == 0) bulk_wait_all();
    return;
  }
  typedef XReg<T, NF> XR;
  typedef typename XR::C RC;
  C* res = xfft<-1, T, TC, NF, !DFS, false>(X, Y, px, tw);
  RC R[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int e = threadIdx.x + j * 256;
    if (e < nel) R[j] = reinterpret_cast<const RC*>(res)[e];
  }
  C* prev = nullptr;  // the buffer the last tensor store reads
  for (int a = 0; a < M; ++a) {
    const int b = a & 1;
    ok = mbar_wait(&bar[b], (unsigned)((a >> 1) & 1), status);
    if (!__syncthreads_and(ok)) break;
    const bool odd = weight_is_odd(a);
    // fill the buffer the previous store does not read; the transform's first
    // stage writes the other one, so that store must have read it by then
    C* in = (prev == X) ? Y : X;
    C* other = (in == X) ? Y : X;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int e = threadIdx.x + j * 256;
      if (e < nel) reinterpret_cast<RC*>(in)[e] = mul_weight(R[j], XR::template load_weight<DFS>(Wst(b), e), odd);
    }
    if (threadIdx.x == 0) bulk_wait_read();
    __syncthreads();
    if (threadIdx.x == 0 && a + 2 < M) {
      mbar_arrive_expect_tx(&bar[b], (unsigned)wbytes);
      tma_load_3d(Wst(b), &mapW, col0, 0, a + 2, &bar[b]);
    }
    C* r2 = xfft<+1, T, TC, NF, false, !DFS>(in, other, px, tw);
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store_3d(&mapC, col0 * E, 0, a, r2);
      bulk_commit();
    }
    prev = r2;
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

// E = IFFT_x(sum_a FFT_x(D[a]) . w_a + FFT_x(A) . w_att); sources are
// double-buffered (spectrum tile + weight tile per stage), the sum lives in
// registers. With the mean field, the Parseval sum for its energy goes to part.
template <class T, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256, 2) k_xbackconv_tma(const __grid_constant__ CUtensorMap mapD, const __grid_constant__ CUtensorMap mapW,
                                                       const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapWatt,
                                                       const __grid_constant__ CUtensorMap mapE, int M, int with_mf, Dims d, FFTPlan px,
                                                       const typename Cx<T>::type* __restrict__ tw, double* __restrict__ part,
                                                       unsigned* __restrict__ status) {
  typedef typename Cx<T>::type C;
  constexpr int TC = TileCols<T>::value, E = ElemsPerComplex<T>::value;
  constexpr int PER = TC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* sm = aligned_smem(smem_raw);
  const int n = px.n;
  const size_t tile_bytes = (size_t)n * TC * sizeof(C), wbytes = (size_t)n * TC * sizeof(T);
  const size_t tb = r128(tile_bytes), wb = r128(wbytes);
  auto Dst = [&](int b) { return reinterpret_cast<C*>(sm + (size_t)b * tb); };  // not pointer arrays (local memory)
  C* Y = reinterpret_cast<C*>(sm + 2 * tb);
  auto Wst = [&](int b) { return reinterpret_cast<T*>(sm + 3 * tb + (size_t)b * wb); };
  __shared__ __align__(8) uint64_t bar[2];
  const int col0 = blockIdx.x * TC;
  const int nel = n * TC;
  const int nsrc = M + (with_mf ? 1 : 0);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int a, int b) {
    mbar_arrive_expect_tx(&bar[b], (unsigned)(tile_bytes + wbytes));
    if (a < M) {
      tma_load_3d(Dst(b), &mapD, col0 * E, 0, a, &bar[b]);
      tma_load_3d(Wst(b), &mapW, col0, 0, a, &bar[b]);
    } else {
      tma_load_3d(Dst(b), &mapA, col0 * E, 0, 0, &bar[b]);
      tma_load_3d(Wst(b), &mapWatt, col0, 0, 0, &bar[b]);
    }
  };
  if (threadIdx.x == 0)
    for (int b = 0; b < 2 && b < nsrc; ++b) issue(b, b);
  typedef XReg<T, NF> XR;
  typedef typename XR::C RC;
  RC S[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) S[j] = XR::zero();
  KahanT<T> pars;  // the mean-field energy by Parseval: compensated in the bulk precision, merged in FP64
  dfs parsd = dfs(0);  // the same in df64 (DFS)
  bool ok = true;
  for (int a = 0; a < nsrc; ++a) {
    const int b = a & 1;
    ok = mbar_wait(&bar[b], (unsigned)((a >> 1) & 1), status);
    if (!__syncthreads_and(ok)) break;
    C* res = xfft<-1, T, TC, NF, !DFS, false>(Dst(b), Y, px, tw);
    const bool is_mf = (a == M);
    const bool odd = !is_mf && weight_is_odd(a);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int e = threadIdx.x + j * 256;
      if (e < nel) {
        const RC z = reinterpret_cast<const RC*>(res)[e];
        const typename XR::W wv = XR::template load_weight<DFS>(Wst(b), e);
        if constexpr (XR::df) S[j] = dfcl_add(S[j], mul_weight(z, wv, odd));  // summed unnormalised, renormalised once below
        else S[j] = cadd(S[j], mul_weight(z, wv, odd));
        if (is_mf) {
          const int col = col0 + (e % TC);
          const int kz = col % d.pz;
          if (kz < d.nzc && col < d.ny * d.pz) {
            const bool one = (kz == 0 || 2 * kz == d.nz);
            if constexpr (XR::df && DFS) {
              const dfs q = (z.x * z.x + z.y * z.y) * wv;
              parsd += one ? q : q + q;
            } else {
              const T mult = one ? (T)1 : (T)2;
              const T zx = XR::re(z), zy = XR::im(z);
              pars.add(mult * (zx * zx + zy * zy) * Wst(b)[e]);
            }
          }
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && a + 2 < nsrc) issue(a + 2, b);
  }
  if constexpr (XR::df && DFS) pars.add((T)dfs_join(parsd));
  if (part) block_kahan_store<1>(&pars, part, blockIdx.x);
  if (!__syncthreads_and(ok)) {
    if (threadIdx.x == 0) bulk_wait_all();
    return;
  }
  C* X = Dst(0);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int e = threadIdx.x + j * 256;
    if (e < nel) {
      if constexpr (XR::df) {  // renormalised once: a transform's first stage keeps its error small on normalised pairs
        S[j].x = df_renorm(S[j].x);
        S[j].y = df_renorm(S[j].y);
      }
      reinterpret_cast<RC*>(X)[e] = S[j];
    }
  }
  C* r2 = xfft<+1, T, TC, NF, false, !DFS>(X, Y, px, tw);
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    tma_store_3d(&mapE, col0 * E, 0, 0, r2);
    bulk_commit();
    bulk_wait_all();
  }
}

}  // namespace cdft

namespace cdft {

// ------------------------------------------------- fused Phi on z rows ---
// Persistent: each block walks groups of RB consecutive rows (x, y). One
// tensor copy brings the group's M field rows ({pz*E, rows, M}, box
// {pz*E, RB, M}) while an earlier group is computed (PhiBufs input buffers:
// the next group's copy is issued as soon as a buffer has been unpacked). The M rows of a (x, y)
// are paired into complex lines (PhiPack); a group is a [nz][L] tile of L lines,
// transformed column-wise (line-fastest, conflict-free):
// c2r (z), Phi and dPhi per point, r2c (z), then the M derivative rows are
// stored over the inputs.
// threads per block of the fused Phi pass (512 threads with two blocks per SM
// measured no faster in FP32 than 256)
template <class T> struct PhiThreads { static constexpr int value = 256; };
// input buffers of the fused Phi pass. One suffices when a group's compute
// (two FFTs and the functional, ~10 us) outlasts its load (24 KB): the load of
// the next group is issued as soon as the current one has been unpacked. In
// FP32 that frees the shared memory for a third resident block per SM.
template <class T> struct PhiBufs { static constexpr int value = sizeof(T) == 4 ? 1 : 2; };
// minimum resident blocks the register allocation must allow
template <class T> struct PhiMinBlocks { static constexpr int value = sizeof(T) == 4 ? 3 : 2; };

// How a row group's M field rows share complex lines for the z transforms: two fields
// per line (real part the even field a, imaginary part a + 1). With CROSS, M odd and RB
// even, the last field of rows 2j and 2j + 1 shares one line (real part row 2j), so no
// line is half empty: M = 11 takes 5 RB + RB / 2 lines instead of 6 RB. It pays in FP64,
// where the FP64 pipe bounds the pass (1/12 fewer transforms); the FP32 pass is bound by
// instruction issue and measured slower with the extra index work, so it keeps 6 RB.
template <int M, int RB, bool CROSS = true> struct PhiPack {
  static constexpr bool cross = CROSS && (M % 2 == 1) && (RB % 2 == 0);
  static constexpr int per_row = cross ? M / 2 : (M + 1) / 2;  // lines holding fields of one row only
  static constexpr int L = per_row * RB + (cross ? RB / 2 : 0);
  // the line and the component (0 real, 1 imaginary) of field a of row r
  __host__ __device__ static constexpr int line(int r, int a) { return (cross && a == M - 1) ? per_row * RB + r / 2 : r * per_row + a / 2; }
  __host__ __device__ static constexpr int comp(int r, int a) { return (cross && a == M - 1) ? (r & 1) : (a & 1); }
  // the field a (-1: none) and row r of a line's real (h = 0) or imaginary (h = 1) part
  __host__ __device__ static constexpr void source(int l, int h, int& a, int& r) {
    if (l < per_row * RB) {
      r = l / per_row;
      a = 2 * (l - r * per_row) + h;
      if (a >= M) a = -1;
    } else {
      r = 2 * (l - per_row * RB) + h;
      a = M - 1;
    }
  }
};
// the FP64 256-point instance reads its row groups in two tensor copies (a row of 264
// doubles exceeds the 256-element box)
template <class T, int NF> struct PhiSplit { static constexpr bool value = sizeof(T) == 8 && NF == 256; };
// one row of df64 spectra in the Phi pass's input buffer: element k is p0[k] below `half`,
// else p1[k - half] (the second box of a split row group)
struct DfRow {
  const dfc* p0 = nullptr;
  const dfc* p1 = nullptr;
  int half = 0;
  __device__ __forceinline__ dfc operator[](int k) const { return k < half ? p0[k] : p1[k - half]; }
  __device__ __forceinline__ explicit operator bool() const { return p0 != nullptr; }
};
// PhiPack<M, RB, cross>::L for a runtime M (host side)
inline int phi_lines(int M, int RB, bool cross) { return (cross && M % 2 == 1 && RB % 2 == 0) ? (M / 2) * RB + RB / 2 : ((M + 1) / 2) * RB; }
// the Phi pass pairs across rows in FP64 only
template <class T> struct PhiCross { static constexpr bool value = sizeof(T) == 8; };
template <class T> __device__ __forceinline__ T cpart(const typename Cx<T>::type& z, int h) { return h ? z.y : z.x; }
template <class T> __device__ __forceinline__ void set_cpart(typename Cx<T>::type* z, int h, T v) {
  if (h) z->y = v;
  else z->x = v;
}

// MODE selects what the pass does per point after the z c2r:
//   kPhiEval  Phi and dPhi (the evaluation; Phi summed into part);
//   kPhiHess  the z-row step of the Hessian-vector product (FMT::add_second_derivative,
//             src/FMT.cpp:437-567): Cf holds the convolutions of v, NA the M weighted densities
//             of the linearisation state in real space (M x N); the folded (d2Phi).Psi replaces
//             Psi;
//   kPhiStoreN  stores the M weighted densities into NA (M x N) and ends there: the set-up of
//             the Hessian products at a state (no r2c, Cf left as it is);
//   kPhiAO    kPhiEval for an FMT_AO_Species, which also stores the M weighted densities
//             into NA and the derivative fields folded with the polymer diameter (inverse
//             iph, iph^2 = iph2) into XA, both M x N in real space, for the AO passes.
// kPhiEval and kPhiAO sum energies and check eta (part and those status bits unused otherwise).
constexpr int kPhiEval = 0, kPhiHess = 1, kPhiStoreN = 2, kPhiAO = 3;
template <class T, int MODEL, int RB, int NF = 0, int MODE = kPhiEval>
__global__ void __launch_bounds__(PhiThreads<T>::value, (MODE == kPhiHess || MODE == kPhiAO) ? 2 : PhiMinBlocks<T>::value) k_phi_rows_tma(const __grid_constant__ CUtensorMap mapR, typename Cx<T>::type* __restrict__ Cf,
                                                      Dims d, FFTPlan pz_plan, const typename Cx<T>::type* __restrict__ tw, T hsd, T esA,
                                                      T esB, double* __restrict__ part, unsigned* __restrict__ status,
                                                      T* __restrict__ NA = nullptr, T* __restrict__ XA = nullptr, T iph = 0, T iph2 = 0) {
  typedef typename Cx<T>::type C;
  constexpr int M = ModelTraits<MODEL>::M;
  typedef PhiPack<M, RB, PhiCross<T>::value> PK;
  const T ih = (T)(1.0 / (double)hsd), ih2 = (T)(1.0 / ((double)hsd * (double)hsd));
  // FP64 with a compile-time plan: the spectra in HBM are double-float (the evaluator runs
  // this instance only when every pass keeps them so), the tile holds df64 values from the
  // unpacking to the Hermitian split (both transforms on the FP32 pipe), and the
  // evaluation's functional runs in df64 too, its f-functions of eta in FP64 (fmt_f_df);
  // the other modes and RSLT take FP64 values per point (getv / setv convert).
  constexpr bool DF = kDf64Transforms && std::is_same<T, double>::value && NF > 0;
  constexpr bool DF_FUNC = DF && MODE == kPhiEval && MODEL != MODEL_RSLT;
  // the Hessian's per-point step in df64 too: the set-up pass (kPhiStoreN) then stores the
  // weighted densities NA as df64 pairs (8 bytes, like the doubles they replace)
  constexpr bool DF_HESS = DF && (MODE == kPhiHess || MODE == kPhiStoreN) && MODEL != MODEL_RSLT;
  auto getv = [&](const C* buf, int i, int h) -> T {
    if constexpr (DF) {
      const dfc z = reinterpret_cast<const dfc*>(buf)[i];
      return (T)dfs_join(h ? z.y : z.x);
    } else {
      return cpart<T>(buf[i], h);
    }
  };
  auto setv = [&](C* buf, int i, int h, T v) {
    if constexpr (DF) {
      dfc* z = reinterpret_cast<dfc*>(buf) + i;
      (h ? z->y : z->x) = dfs_split((double)v);
    } else {
      set_cpart<T>(&buf[i], h, v);
    }
  };
  constexpr int L = PK::L;
  constexpr int LPd = L | 1;  // odd row pitch: the per-point loops stride rows without bank conflicts
  constexpr int E = ElemsPerComplex<T>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* sm = aligned_smem(smem_raw);
  // with a compile-time plan the row length is a constant too (the divisions below fold)
  const int nz = NF > 0 ? NF : d.nz, nzc = NF > 0 ? NF / 2 + 1 : d.nzc, pz = d.pz;
  // A 256-point FP64 row (132 complex, 264 doubles) is wider than a tensor copy's 256-element
  // box: the group then arrives in two boxes, the first and second half of every row, each
  // box a [M][RB][pz / 2] block (the second 128-byte aligned).
  constexpr bool SPLIT = PhiSplit<T, NF>::value;
  const int rowc = SPLIT ? pz / 2 : pz;  // complex values per row in one block
  const size_t in_bytes = (size_t)M * RB * pz * sizeof(C), hb = r128((size_t)M * RB * rowc * sizeof(C));
  const size_t ib = SPLIT ? 2 * hb : r128(in_bytes);
  const size_t zb = r128((size_t)nz * LPd * sizeof(C));
  constexpr int NB = PhiBufs<T>::value;
  auto In = [&](int b) { return reinterpret_cast<C*>(sm + (size_t)(b % NB) * ib); };  // not a pointer array (local memory)
  C* Z0 = reinterpret_cast<C*>(sm + NB * ib);
  C* Z1 = reinterpret_cast<C*>(sm + NB * ib + zb);
  __shared__ __align__(8) uint64_t bar[NB];
  const long ngroup = (d.rows + RB - 1) / RB;
  if constexpr (DF_FUNC || (DF_HESS && MODE == kPhiHess)) df_log_table_init(threadIdx.x, blockDim.x);  // read after the barrier below
  if (threadIdx.x == 0) {
#pragma unroll
    for (int b = 0; b < NB; ++b) mbar_init(&bar[b], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](long g, int b) {
    mbar_arrive_expect_tx(&bar[b], (unsigned)in_bytes);
    tma_load_3d(In(b), &mapR, 0, (int)(g * RB), 0, &bar[b]);
    if constexpr (SPLIT) tma_load_3d(reinterpret_cast<unsigned char*>(In(b)) + hb, &mapR, rowc * E, (int)(g * RB), 0, &bar[b]);
  };
  if (threadIdx.x == 0)
    for (int b = 0; b < NB; ++b) {
      const long g = blockIdx.x + (long)b * gridDim.x;
      if (g < ngroup) issue(g, b);
    }
  KahanT<T> psum;
  dfs psd = dfs(0);  // the df64 functional's sum (a thread's points), joined once
  struct DfParams { dfs x, y, z, w; } dfi;  // 1/hsd, 1/hsd^2, esA, esB in df64
  if constexpr (DF_FUNC || DF_HESS) dfi = {dfs_split((double)ih), dfs_split((double)ih2), dfs_split((double)esA), dfs_split((double)esB)};
  unsigned st = 0;
  bool ok = true;
  for (long it = 0;; ++it) {
    const long g = blockIdx.x + it * gridDim.x;
    if (g >= ngroup) break;
    const int b = (int)(it % NB);
    ok = mbar_wait(&bar[b], (unsigned)((it / NB) & 1), status);
    if (!__syncthreads_and(ok)) break;
    const long row0 = g * RB;
    const C* in = In(b);
    // packed Hermitian spectra (PhiPack's lines), element k of [nz][L]
    for (int e = threadIdx.x; e < nz * L; e += blockDim.x) {
      const int line = e % L, k = e / L;
      int aA, rA, aB, rB;
      PK::source(line, 0, aA, rA);
      PK::source(line, 1, aB, rB);
      if constexpr (DF) {
        const dfc* h0 = reinterpret_cast<const dfc*>(in);
        const dfc* h1 = reinterpret_cast<const dfc*>(reinterpret_cast<const unsigned char*>(in) + hb);
        const DfRow Ar{h0 + ((size_t)aA * RB + rA) * rowc, h1 + ((size_t)aA * RB + rA) * rowc, rowc};
        const DfRow Br = aB >= 0 ? DfRow{h0 + ((size_t)aB * RB + rB) * rowc, h1 + ((size_t)aB * RB + rB) * rowc, rowc} : DfRow{};
        reinterpret_cast<dfc*>(Z0)[k * LPd + line] = pair_spectrum_df(Ar, Br, k, nz);
      } else {
        const C* Arow = in + ((size_t)aA * RB + rA) * pz;
        const C* Brow = aB >= 0 ? in + ((size_t)aB * RB + rB) * pz : nullptr;
        Z0[k * LPd + line] = pair_spectrum<T>(Arow, Brow, k, nz);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // In(b) consumed: bring the group NB steps ahead
      const long gn = g + (long)NB * gridDim.x;
      if (gn < ngroup) issue(gn, b);
    }
    C* res;
    if constexpr (DF) res = tile_fft_fixed_df<+1, L, LPd, NF, PhiThreads<T>::value, false, false>(Z0, Z1, reinterpret_cast<const dfc*>(tw + fx_table_len(NF)));
    else res = tfft<+1, T, L, LPd, NF, PhiThreads<T>::value>(Z0, Z1, pz_plan, tw);
    if constexpr (MODE == kPhiStoreN) {
      for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
        const int k = e % nz, r = e / nz;
        if (row0 + r >= d.rows) continue;
#pragma unroll
        for (int a = 0; a < M; ++a) {
          if constexpr (DF_HESS) {  // df64 pairs, read back by the Hessian's df64 step
            const dfc z = reinterpret_cast<const dfc*>(res)[k * LPd + PK::line(r, a)];
            reinterpret_cast<dfs*>(NA)[(long)a * d.N + (row0 + r) * nz + k] = PK::comp(r, a) ? z.y : z.x;
          } else {
            NA[(long)a * d.N + (row0 + r) * nz + k] = getv(res, k * LPd + PK::line(r, a), PK::comp(r, a));
          }
        }
      }
      __syncthreads();
      continue;
    }
    C* oth = (res == Z0) ? Z1 : Z0;
    for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
      const int k = e % nz, r = e / nz;
      if (row0 + r >= d.rows) {  // a row past the end: zeros into its slots (a line may pair it with a live row)
#pragma unroll
        for (int a = 0; a < M; ++a) setv(oth, k * LPd + PK::line(r, a), PK::comp(r, a), (T)0);
        continue;
      }
      if constexpr (DF_FUNC) {  // the functional in df64, values kept in df64 both ways
        const dfc* rd = reinterpret_cast<const dfc*>(res);
        dfc* od = reinterpret_cast<dfc*>(oth);
        dfs nw[11];
#pragma unroll
        for (int a = 0; a < M; ++a) {
          const dfc z = rd[k * LPd + PK::line(r, a)];
          nw[a] = PK::comp(r, a) ? z.y : z.x;
        }
        if ((dfs(1) - nw[0]).h < 0.f) st |= 1u;  // eta > 1 (nw[0] is eta until the functional overwrites it)
        // the functional in the lazy df64 arithmetic (dfl): its derivatives go straight into
        // the forward transform's first stage, which takes unnormalised pairs
        dfl nl[11];
#pragma unroll
        for (int a = 0; a < M; ++a) nl[a] = dfl(nw[a]);
        const dfs phi = fmt_phi_point<dfl, MODEL>(nl, dfl(dfi.x), dfl(dfi.y), dfl(dfi.z), dfl(dfi.w)).norm();
        if (!isfinite(phi.h)) st |= 2u;
        psd += phi;
#pragma unroll
        for (int a = 0; a < M; ++a) nw[a] = nl[a].raw();
#pragma unroll
        for (int p = 0; p < PK::per_row; ++p) {
          dfc z;
          z.x = nw[2 * p];
          z.y = (2 * p + 1 < M) ? nw[2 * p + 1] : dfs(0);
          od[k * LPd + r * PK::per_row + p] = z;
        }
        if constexpr (PK::cross) {
          dfc* z = od + k * LPd + PK::line(r, M - 1);
          (PK::comp(r, M - 1) ? z->y : z->x) = nw[M - 1];
        }
        continue;
      }
      if constexpr (DF_HESS && MODE == kPhiHess) {  // (d2Phi).Psi per point in df64, NA stored as df64 pairs
        const dfc* rd = reinterpret_cast<const dfc*>(res);
        dfc* od = reinterpret_cast<dfc*>(oth);
        const dfs* nad = reinterpret_cast<const dfs*>(NA);
        dfs nw[11], nd[11];
#pragma unroll
        for (int a = 0; a < M; ++a) {
          const dfc z = rd[k * LPd + PK::line(r, a)];
          nw[a] = PK::comp(r, a) ? z.y : z.x;
          nd[a] = nad[(long)a * d.N + (row0 + r) * nz + k];
        }
        {  // in the lazy df64 arithmetic, as the functional above
          dfl ndl[11], nwl[11];
#pragma unroll
          for (int a = 0; a < M; ++a) {
            ndl[a] = dfl(nd[a]);
            nwl[a] = dfl(nw[a]);
          }
          const dfl ih(dfi.x), ih2(dfi.y);
          fmt_d2phi_dot_point<dfl, MODEL>(ndl, nwl, ih, ih2, dfl(dfi.z), dfl(dfi.w), ih, ih2);
#pragma unroll
          for (int a = 0; a < M; ++a) nw[a] = nwl[a].raw();
        }
#pragma unroll
        for (int p = 0; p < PK::per_row; ++p) {
          dfc z;
          z.x = nw[2 * p];
          z.y = (2 * p + 1 < M) ? nw[2 * p + 1] : dfs(0);
          od[k * LPd + r * PK::per_row + p] = z;
        }
        if constexpr (PK::cross) {
          dfc* z = od + k * LPd + PK::line(r, M - 1);
          (PK::comp(r, M - 1) ? z->y : z->x) = nw[M - 1];
        }
        continue;
      }
      T nv[11];
#pragma unroll
      for (int a = 0; a < M; ++a) nv[a] = getv(res, k * LPd + PK::line(r, a), PK::comp(r, a));
      if constexpr (MODE == kPhiHess) {
        T nd[11];
#pragma unroll
        for (int a = 0; a < M; ++a) nd[a] = NA[(long)a * d.N + (row0 + r) * nz + k];
        fmt_d2phi_dot_point<T, MODEL>(nd, nv, ih, ih2, esA, esB, ih, ih2);
      } else {
        const long idx = (row0 + r) * nz + k;
        if constexpr (MODE == kPhiAO) {
#pragma unroll
          for (int a = 0; a < M; ++a) NA[(long)a * d.N + idx] = nv[a];
        }
        T ao4[4];
        const T eta = nv[0];
        const T phi = fmt_phi_point<T, MODEL>(nv, ih, ih2, esA, esB, MODE == kPhiAO ? ao4 : nullptr, iph, iph2);
        if (eta > (T)0.5 && (T)1 - eta < (T)0) st |= 1u;
        if (!isfinite(phi)) st |= 2u;
        psum.add(phi);
        if constexpr (MODE == kPhiAO) {
#pragma unroll
          for (int a = 0; a < M; ++a) XA[(long)a * d.N + idx] = (a >= 1 && a <= 4) ? ao4[a - 1] : nv[a];
        }
      }
#pragma unroll
      for (int p = 0; p < PK::per_row; ++p) {
        setv(oth, k * LPd + r * PK::per_row + p, 0, nv[2 * p]);
        setv(oth, k * LPd + r * PK::per_row + p, 1, (2 * p + 1 < M) ? nv[2 * p + 1] : (T)0);
      }
      if constexpr (PK::cross) setv(oth, k * LPd + PK::line(r, M - 1), PK::comp(r, M - 1), nv[M - 1]);
    }
    C* res2;
    if constexpr (DF) res2 = tile_fft_fixed_df<-1, L, LPd, NF, PhiThreads<T>::value, false, false>(oth, res, reinterpret_cast<const dfc*>(tw + fx_table_len(NF)));
    else res2 = tfft<-1, T, L, LPd, NF, PhiThreads<T>::value>(oth, res, pz_plan, tw);
    for (int e = threadIdx.x; e < L * nzc; e += blockDim.x) {
      const int k = e % nzc, line = e / nzc;
      int aA, rA, aB, rB;
      PK::source(line, 0, aA, rA);
      PK::source(line, 1, aB, rB);
      if constexpr (DF) {  // the split in df64, the spectra stored as df64
        const dfc* rd = reinterpret_cast<const dfc*>(res2);
        const dfc Z = rd[k * LPd + line], W = rd[(k == 0 ? 0 : nz - k) * LPd + line];
        dfc* o = reinterpret_cast<dfc*>(Cf);
        if (row0 + rA < d.rows) o[(long)aA * d.Nc + (row0 + rA) * pz + k] = dfc{df_half(Z.x + W.x), df_half(Z.y - W.y)};
        if (aB >= 0 && row0 + rB < d.rows) o[(long)aB * d.Nc + (row0 + rB) * pz + k] = dfc{df_half(Z.y + W.y), df_half(W.x - Z.x)};
      } else {
        const C Z = res2[k * LPd + line];
        const C W = res2[(k == 0 ? 0 : nz - k) * LPd + line];
        if (row0 + rA < d.rows) Cf[(long)aA * d.Nc + (row0 + rA) * pz + k] = mk<T>((T)0.5 * (Z.x + W.x), (T)0.5 * (Z.y - W.y));
        if (aB >= 0 && row0 + rB < d.rows) Cf[(long)aB * d.Nc + (row0 + rB) * pz + k] = mk<T>((T)0.5 * (Z.y + W.y), (T)0.5 * (W.x - Z.x));
      }
    }
    __syncthreads();
  }
  if constexpr (MODE == kPhiEval || MODE == kPhiAO) {
    if (st) atomicOr(status, st);
    if constexpr (DF_FUNC) psum.add((T)dfs_join(psd));
    block_kahan_store<1>(&psum, part, blockIdx.x);
  }
  (void)E;
}

}  // namespace cdft

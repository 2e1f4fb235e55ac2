// Device kernels of the F+dF evaluation (sm_103a). Layout in HBM follows the
// reference's Lattice (include/Lattice.h:120-134): real fields row-major
// pos = k + Nz*(j + Ny*i); half spectra kpos = kz + Nzc*(ky + Ny*kx) with
// Nzc = Nz/2 + 1 (FFTW r2c layout). Transforms are unnormalised.
//
// Internally the half spectrum's rows are padded to pz = round_up(Nzc, 4)
// (kpos = kz + pz*(ky + Ny*kx)) so that every tensor-copy stride is a multiple
// of 16 bytes; columns kz >= Nzc are padding and carry no data.
//
// Pass structure of one evaluation (T = float or double):
//   rows_r2c     rho (f64) -> A            z-axis r2c, two rows per complex FFT
//   cols_fft(y)  A                          y-axis forward
//   xconv        A -> C[a], a < M          x-axis forward, x w_a, x-axis inverse
//   cols_fft(y)  C[a]                       y-axis inverse (batched over a)
//   phi_rows     C[a] -> D[a] (in place)   z-axis c2r, Phi/dPhi, z-axis r2c
//   cols_fft(y)  D[a]                       y-axis forward (batched)
//   xbackconv    D[a], A -> E              x-axis forward, sum_a D~ w_a (+ rho~ w_att),
//                                           x-axis inverse
//   cols_fft(y)  E                          y-axis inverse
//   final_rows   E, rho -> dF (f64)         z-axis c2r + ideal/external terms
#pragma once
#include "cdft_fft.cuh"
#include "cdft_fft_df.cuh"
#include "cdft_phi.cuh"
#include "cdft_convert.cuh"

namespace cdft {

struct Dims {
  int nx, ny, nz, nzc;
  long N, Nc;  // Nc = nx*ny*pz: spectra are stored with a padded row pitch
  long rows;   // nx*ny
  int pz;      // row pitch of the half spectrum: nzc rounded up to a multiple of 4
};

// ----------------------------------------------------------- reductions ---
struct Acc {  // Neumaier compensated FP64 accumulator
  double s, c;
  __device__ __forceinline__ void init() { s = 0; c = 0; }
  __device__ __forceinline__ void add(double v) {
    double t = s + v;
    if (fabs(s) >= fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ void merge(double s2, double c2) { add(s2); c += c2; }
};

// Block-wide merge of NV accumulators; thread 0 writes (s, c) pairs to
// out[(blockIdx.x * NV + v) * 2 + {0,1}] (out indexed by the linear block id).
template <int NV>
__device__ __forceinline__ void block_reduce_store(Acc* acc, double* out, long block_id) {
  __shared__ double red[32][NV][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double s2 = __shfl_down_sync(0xffffffffu, acc[v].s, o);
      double c2 = __shfl_down_sync(0xffffffffu, acc[v].c, o);
      acc[v].merge(s2, c2);
    }
    if (lane == 0) { red[warp][v][0] = acc[v].s; red[warp][v][1] = acc[v].c; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int v = 0; v < NV; ++v) {
      Acc t;
      t.init();
      for (int w = 0; w < nw; ++w) t.merge(red[w][v][0], red[w][v][1]);
      out[(block_id * NV + v) * 2 + 0] = t.s;
      out[(block_id * NV + v) * 2 + 1] = t.c;
    }
  }
}

// Block-wide plain FP64 sum of NV per-thread partials (a thread's partial
// covers only a few points); thread 0 stores (sum, 0) pairs in the layout of
// block_reduce_store. The compensated merge across blocks is k_finish_reduce.
template <int NV>
__device__ __forceinline__ void block_sum_store(double* v, double* out, long block_id) {
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0) red[warp][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    const int k = threadIdx.x;
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][k];
    out[(block_id * NV + k) * 2 + 0] = t;
    out[(block_id * NV + k) * 2 + 1] = 0.0;
  }
}

// value of type D from type S: the integer-pipe conversions between FP64 and FP32, plain casts otherwise
template <class D, class S>
__device__ __forceinline__ D conv(S x) { return (D)x; }
template <>
__device__ __forceinline__ float conv<float, double>(double x) { return cvt_f32(x); }
template <>
__device__ __forceinline__ double conv<double, float>(float x) { return cvt_f64(x); }

// Kahan-compensated running sum in the bulk precision (a thread's few points).
template <class T>
struct KahanT {
  T s = 0, c = 0;
  __device__ __forceinline__ void add(T v) {
    const T y = v - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
// FP64 per-thread partials are plain sums: a thread adds only a few dozen terms (its
// rounding error stays near 1e-15 of them), the merges across threads and blocks are the
// compensated ones, and each Kahan step costs three more instructions of GB300's small
// FP64 pipe.
template <>
struct KahanT<double> {
  double s = 0, c = 0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double value() const { return s; }
};

// Block-wide merge of NV per-thread Kahan partials, stored like block_sum_store.
// FP32 partials merge across the warp in FP32 with error-free sums (Knuth's
// TwoSum: the rounding error of every merge goes into the compensation term),
// so the small FP64 unit sees one conversion and one add per warp and value
// instead of a conversion and five adds per thread. FP64 partials take the
// plain FP64 path.
template <int NV, class T>
__device__ __forceinline__ void block_kahan_store(const KahanT<T>* ks, double* out, long block_id) {
  if constexpr (sizeof(T) == 8) {
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = ks[k].value();
    block_sum_store<NV>(v, out, block_id);
  } else {
    __shared__ double red[32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      float s = ks[k].s, c = ks[k].c;  // value s - c
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, s, o);
        const float c2 = __shfl_down_sync(0xffffffffu, c, o);
        const float t = s + s2;
        const float bb = t - s;
        const float e = (s - (t - bb)) + (s2 - bb);  // s + s2 = t + e exactly
        c = (c + c2) - e;
        s = t;
      }
      if (lane == 0) red[warp][k] = cvt_f64(s) - cvt_f64(c);
    }
    __syncthreads();
    if (threadIdx.x < NV) {
      const int k = threadIdx.x;
      double t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][k];
      out[(block_id * NV + k) * 2 + 0] = t;
      out[(block_id * NV + k) * 2 + 1] = 0.0;
    }
  }
}

// Block-wide (sum of squares, max) of the per-thread partials q (Kahan) and
// mx; thread 0 stores out[2 * block_id] = sum, out[2 * block_id + 1] = max,
// the layout the dF-norm finish reads. FP32 partials merge in FP32 as in
// block_kahan_store.
template <class T>
__device__ __forceinline__ void block_norms_store(const KahanT<T>& q, T mx, double* out, long block_id) {
  __shared__ double red_s[32], red_m[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (sizeof(T) == 8) {
    double v = q.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_down_sync(0xffffffffu, v, o);
      const double m2 = __shfl_down_sync(0xffffffffu, mx, o);
      mx = m2 > mx ? m2 : mx;
    }
    if (lane == 0) { red_s[warp] = v; red_m[warp] = mx; }
  } else {
    float s = q.s, c = q.c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_down_sync(0xffffffffu, s, o);
      const float c2 = __shfl_down_sync(0xffffffffu, c, o);
      const float m2 = __shfl_down_sync(0xffffffffu, mx, o);
      const float t = s + s2;
      const float bb = t - s;
      const float e = (s - (t - bb)) + (s2 - bb);
      c = (c + c2) - e;
      s = t;
      mx = m2 > mx ? m2 : mx;
    }
    if (lane == 0) { red_s[warp] = cvt_f64(s) - cvt_f64(c); red_m[warp] = cvt_f64(mx); }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0, m = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t += red_s[w];
      m = red_m[w] > m ? red_m[w] : m;
    }
    out[2 * block_id] = t;
    out[2 * block_id + 1] = m;
  }
}

// Sums nblk partial (s, c) pairs of NV values in a fixed order: out[v] = total.
__global__ void k_finish_reduce(const double* __restrict__ part, long nblk, int nv, double* __restrict__ out);

// ------------------------------------------------------------ row passes ---
// FP64 spectra kept in double-float between passes: an instance with DFS (FP64, compile-time
// plan) reads and writes each complex value as a dfc where the others use a double2.
template <class T, int NF, bool DFS> struct DfSpectra {
  static constexpr bool value = DFS && kDf64Transforms && sizeof(T) == 8 && NF > 0;
};

// z-axis r2c: rows of a real field (SRC = double or T) to half spectra.
// Each block owns RB row pairs; pair r packs rows (2r, 2r+1) as re/im.
template <class T, class SRC, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256) k_rows_r2c(const SRC* __restrict__ in, typename Cx<T>::type* __restrict__ out, Dims d,
                                                  FFTPlan pz, const typename Cx<T>::type* __restrict__ tw, int RB) {
  typedef typename Cx<T>::type C;
  constexpr bool DS = DfSpectra<T, NF, DFS>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* b0 = reinterpret_cast<C*>(smem_raw);
  const int nz = NF > 0 ? NF : d.nz, LP = nz + 1;
  C* b1 = b0 + RB * LP;
  const long pair0 = (long)blockIdx.x * RB;
  // unrolled so that several rows' loads are in flight before their shared stores
#pragma unroll 4
  for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
    const int r = e / nz, k = e - r * nz;
    const long ra = 2 * (pair0 + r), rb = ra + 1;
    T va = 0, vb = 0;
    if (ra < d.rows) va = conv<T>(in[ra * nz + k]);
    if (rb < d.rows) vb = conv<T>(in[rb * nz + k]);
    b0[r * LP + k] = mk<T>(va, vb);
  }
  C* res = rows_fft<-1, T, NF, true, !DS>(b0, b1, RB, LP, pz, tw);
  const int nzc = NF > 0 ? NF / 2 + 1 : d.nzc;
  for (int e = threadIdx.x; e < RB * nzc; e += blockDim.x) {
    const int r = e / nzc, k = e - r * nzc;
    const long ra = 2 * (pair0 + r), rb = ra + 1;
    if constexpr (DS) {  // the same split in df64
      const dfc* rd = reinterpret_cast<const dfc*>(res);
      const dfc Z = rd[r * LP + k], W = rd[r * LP + (k == 0 ? 0 : nz - k)];
      dfc* o = reinterpret_cast<dfc*>(out);
      if (ra < d.rows) o[ra * d.pz + k] = dfc{df_half(Z.x + W.x), df_half(Z.y - W.y)};
      if (rb < d.rows) o[rb * d.pz + k] = dfc{df_half(Z.y + W.y), df_half(W.x - Z.x)};
      continue;
    }
    const C Z = res[r * LP + k];
    const C W = res[r * LP + (k == 0 ? 0 : nz - k)];  // Z_{N-k}
    // X = (Z + conj(W))/2, Y = (Z - conj(W))/(2i)
    if (ra < d.rows) out[ra * d.pz + k] = mk<T>((T)0.5 * (Z.x + W.x), (T)0.5 * (Z.y - W.y));
    if (rb < d.rows) out[rb * d.pz + k] = mk<T>((T)0.5 * (Z.y + W.y), (T)0.5 * (W.x - Z.x));
  }
}

// Loads the Hermitian-extended pair spectrum Z_k = A_k + i B_k (k < nz) into a
// shared line, dropping Im of kz = 0 and kz = nz/2 as FFTW's c2r does.
template <class T>
__device__ __forceinline__ typename Cx<T>::type pair_spectrum(const typename Cx<T>::type* __restrict__ A, const typename Cx<T>::type* __restrict__ B,
                                                              int k, int nz) {
  typedef typename Cx<T>::type C;
  const int nzc = nz / 2 + 1;
  C a, b;
  if (k < nzc) {
    a = A ? A[k] : mk<T>(0, 0);
    b = B ? B[k] : mk<T>(0, 0);
    if (k == 0 || 2 * k == nz) { a.y = 0; b.y = 0; }
  } else {
    a = A ? A[nz - k] : mk<T>(0, 0);
    b = B ? B[nz - k] : mk<T>(0, 0);
    a.y = -a.y;
    b.y = -b.y;
  }
  return mk<T>(a.x - b.y, a.y + b.x);
}

// pair_spectrum on double-float spectra (R: a pointer, or a row accessor with [] and bool)
template <class R>
__device__ __forceinline__ dfc pair_spectrum_df(const R& A, const R& B, int k, int nz) {
  const int nzc = nz / 2 + 1;
  const dfc zero{dfs(0), dfs(0)};
  dfc a, b;
  if (k < nzc) {
    a = A ? A[k] : zero;
    b = B ? B[k] : zero;
    if (k == 0 || 2 * k == nz) {
      a.y = dfs(0);
      b.y = dfs(0);
    }
  } else {
    a = A ? A[nz - k] : zero;
    b = B ? B[nz - k] : zero;
    a.y = -a.y;
    b.y = -b.y;
  }
  return dfc{a.x - b.y, a.y + b.x};
}

// z-axis c2r: half spectra rows to real rows (DST = double or T), times scale.
template <class T, class DST, int NF = 0>
__global__ void __launch_bounds__(256) k_rows_c2r(const typename Cx<T>::type* __restrict__ in, DST* __restrict__ out, Dims d,
                                                  FFTPlan pz, const typename Cx<T>::type* __restrict__ tw, int RB, T scale) {
  typedef typename Cx<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* b0 = reinterpret_cast<C*>(smem_raw);
  const int nz = d.nz, LP = nz + 1;
  C* b1 = b0 + RB * LP;
  const long pair0 = (long)blockIdx.x * RB;
  for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
    const int r = e / nz, k = e - r * nz;
    const long ra = 2 * (pair0 + r), rb = ra + 1;
    const C* A = ra < d.rows ? in + ra * d.pz : nullptr;
    const C* B = rb < d.rows ? in + rb * d.pz : nullptr;
    b0[r * LP + k] = pair_spectrum<T>(A, B, k, nz);
  }
  C* res = rows_fft<+1, T, NF>(b0, b1, RB, LP, pz, tw);
  for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
    const int r = e / nz, k = e - r * nz;
    const long ra = 2 * (pair0 + r), rb = ra + 1;
    const C z = res[r * LP + k];
    if (ra < d.rows) out[ra * nz + k] = (DST)(z.x * scale);
    if (rb < d.rows) out[rb * nz + k] = (DST)(z.y * scale);
  }
}

// --------------------------------------------------------- column passes ---
// Columns of the half spectrum along x (axis 0, ncol = ny*pz, stride ny*pz)
// or y (axis 1, ncol = nx*nzc, stride pz). A block loads TC consecutive
// columns (coalesced along kz), transforms them in shared memory, stores back.
__device__ __forceinline__ long col_base(int axis, long c, const Dims& d) {
  return axis == 0 ? c : (c / d.nzc) * (long)d.ny * d.pz + (c % d.nzc);
}

template <class T>
__device__ __forceinline__ void load_cols(typename Cx<T>::type* __restrict__ sm, const typename Cx<T>::type* __restrict__ g, int axis,
                                          long c0, long ncol, int n, long stride, int TC, int LP, const Dims& d) {
  for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
    const int c = e % TC, i = e / TC;
    const long col = c0 + c;
    sm[c * LP + i] = (col < ncol) ? g[col_base(axis, col, d) + i * stride] : mk<T>(0, 0);
  }
}
template <class T>
__device__ __forceinline__ void store_cols(const typename Cx<T>::type* __restrict__ sm, typename Cx<T>::type* __restrict__ g, int axis,
                                           long c0, long ncol, int n, long stride, int TC, int LP, const Dims& d) {
  for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
    const int c = e % TC, i = e / TC;
    const long col = c0 + c;
    if (col < ncol) g[col_base(axis, col, d) + i * stride] = sm[c * LP + i];
  }
}

template <class T, int DIR, int NF = 0>
__global__ void __launch_bounds__(256) k_cols_fft(typename Cx<T>::type* __restrict__ data, long field_stride, int axis, Dims d,
                                                  FFTPlan P, const typename Cx<T>::type* __restrict__ tw, int TC) {
  typedef typename Cx<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = P.n, LP = n + 1;
  C* b0 = reinterpret_cast<C*>(smem_raw);
  C* b1 = b0 + TC * LP;
  C* g = data + (long)blockIdx.y * field_stride;
  const long ncol = axis == 0 ? (long)d.ny * d.pz : (long)d.nx * d.nzc;
  const long stride = axis == 0 ? (long)d.ny * d.pz : (long)d.pz;
  const long c0 = (long)blockIdx.x * TC;
  load_cols<T>(b0, g, axis, c0, ncol, n, stride, TC, LP, d);
  C* res = rows_fft<DIR, T, NF>(b0, b1, TC, LP, P, tw);  // the compile-time plan when NF > 0 (df64 in FP64)
  store_cols<T>(res, g, axis, c0, ncol, n, stride, TC, LP, d);
}

// Weight parity: vector weights (a = 2, 3, 4) are odd, so their transform is
// imaginary; all other FMT weights and the mean-field kernel are even (real).
// w holds the one non-zero component per kpos.
__device__ __forceinline__ bool weight_is_odd(int a) { return a >= 2 && a <= 4; }
template <class C, class T>
__device__ __forceinline__ C mul_weight(C z, T w, bool odd) {
  if (odd) return mk<T>(-z.y * w, z.x * w);  // z * (i w)
  return mk<T>(z.x * w, z.y * w);
}

// x-axis pass with the forward weights: C[a] = IFFT_x(FFT_x(A) . w_a).
template <class T>
__global__ void __launch_bounds__(256) k_xconv(const typename Cx<T>::type* __restrict__ A, typename Cx<T>::type* __restrict__ Cout,
                                               const T* __restrict__ w, int M, Dims d, FFTPlan px,
                                               const typename Cx<T>::type* __restrict__ tw, int TC) {
  typedef typename Cx<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = px.n, LP = n + 1;
  C* R = reinterpret_cast<C*>(smem_raw);
  C* b0 = R + TC * LP;
  C* b1 = b0 + TC * LP;
  const long ncol = (long)d.ny * d.pz, stride = ncol;
  const long c0 = (long)blockIdx.x * TC;
  load_cols<T>(b0, A, 0, c0, ncol, n, stride, TC, LP, d);
  C* res = block_fft<-1, T>(b0, b1, TC, LP, px, tw);
  for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
    const int c = e % TC, i = e / TC;
    R[c * LP + i] = res[c * LP + i];
  }
  for (int a = 0; a < M; ++a) {
    const T* wa = w + (long)a * d.Nc;
    const bool odd = weight_is_odd(a);
    __syncthreads();
    for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
      const int c = e % TC, i = e / TC;
      const long col = c0 + c;
      const T wv = col < ncol ? __ldg(wa + i * stride + col) : (T)0;
      b0[c * LP + i] = mul_weight(R[c * LP + i], wv, odd);
    }
    C* r2 = block_fft<+1, T>(b0, b1, TC, LP, px, tw);
    store_cols<T>(r2, Cout + (long)a * d.Nc, 0, c0, ncol, n, stride, TC, LP, d);
  }
}

// x-axis back-convolution: E = IFFT_x(sum_a FFT_x(D[a]) . w_a + FFT_x(A) . w_att).
// With the mean field, each block also accumulates the Parseval sum
// sum_k m(kz) |rho~|^2 w_att (m = 1 on the kz = 0 / Nyquist planes, else 2)
// into part[blockIdx.x] for the interaction energy.
template <class T>
__global__ void __launch_bounds__(256) k_xbackconv(const typename Cx<T>::type* __restrict__ D, const typename Cx<T>::type* __restrict__ A,
                                                   typename Cx<T>::type* __restrict__ E, const T* __restrict__ w,
                                                   const T* __restrict__ watt, int M, Dims d, FFTPlan px,
                                                   const typename Cx<T>::type* __restrict__ tw, int TC, double* __restrict__ part) {
  typedef typename Cx<T>::type C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = px.n, LP = n + 1;
  C* S = reinterpret_cast<C*>(smem_raw);
  C* b0 = S + TC * LP;
  C* b1 = b0 + TC * LP;
  const long ncol = (long)d.ny * d.pz, stride = ncol;
  const long c0 = (long)blockIdx.x * TC;
  for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
    const int c = e % TC, i = e / TC;
    S[c * LP + i] = mk<T>(0, 0);
  }
  const int nsrc = M + (watt ? 1 : 0);
  Acc acc;
  acc.init();
  for (int a = 0; a < nsrc; ++a) {
    const bool is_mf = (a == M);
    const C* src = is_mf ? A : D + (long)a * d.Nc;
    const T* wa = is_mf ? watt : w + (long)a * d.Nc;
    const bool odd = !is_mf && weight_is_odd(a);
    __syncthreads();
    load_cols<T>(b0, src, 0, c0, ncol, n, stride, TC, LP, d);
    C* res = block_fft<-1, T>(b0, b1, TC, LP, px, tw);
    for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
      const int c = e % TC, i = e / TC;
      const long col = c0 + c;
      if (col < ncol) {
        const T wv = __ldg(wa + i * stride + col);
        const C z = res[c * LP + i];
        S[c * LP + i] = cadd(S[c * LP + i], mul_weight(z, wv, odd));
        const int kz = (int)(col % d.pz);
        if (is_mf && kz < d.nzc) {
          const double mult = (kz == 0 || 2 * kz == d.nz) ? 1.0 : 2.0;
          acc.add(mult * ((double)z.x * (double)z.x + (double)z.y * (double)z.y) * (double)wv);
        }
      }
    }
  }
  if (part) block_reduce_store<1>(&acc, part, blockIdx.x);
  __syncthreads();
  for (int e = threadIdx.x; e < TC * n; e += blockDim.x) {
    const int c = e % TC, i = e / TC;
    b0[c * LP + i] = S[c * LP + i];
  }
  C* r2 = block_fft<+1, T>(b0, b1, TC, LP, px, tw);
  store_cols<T>(r2, E, 0, c0, ncol, n, stride, TC, LP, d);
}

// ------------------------------------------------- fused Phi on z rows ---
// For RB rows (x, y): c2r of the M weighted-density rows (fields packed two
// per complex line), Phi and dPhi at every point, r2c of the M derivative
// rows written back over the inputs. Block partial of sum Phi -> part;
// status bit 1: eta > 1 somewhere (Eta_Too_Large), bit 2: non-finite Phi.
template <class T, int MODEL>
__global__ void __launch_bounds__(256) k_phi_rows(typename Cx<T>::type* __restrict__ Cf, Dims d, FFTPlan pz,
                                                  const typename Cx<T>::type* __restrict__ tw, int RB, T hsd, T esA, T esB,
                                                  double* __restrict__ part, unsigned* __restrict__ status) {
  typedef typename Cx<T>::type C;
  constexpr int M = ModelTraits<MODEL>::M;
  constexpr int NP = (M + 1) / 2;
  const T ih = (T)(1.0 / (double)hsd), ih2 = (T)(1.0 / ((double)hsd * (double)hsd));
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nz = d.nz, LP = nz + 1, nzc = d.nzc;
  const int L = NP * RB;
  C* b0 = reinterpret_cast<C*>(smem_raw);
  C* b1 = b0 + L * LP;
  const long row0 = (long)blockIdx.x * RB;
  // line index = r * NP + pair
  for (int e = threadIdx.x; e < L * nz; e += blockDim.x) {
    const int line = e / nz, k = e - line * nz;
    const int r = line / NP, pr = line - r * NP;
    const long row = row0 + r;
    const C* Arow = nullptr;
    const C* Brow = nullptr;
    if (row < d.rows) {
      Arow = Cf + (long)(2 * pr) * d.Nc + row * d.pz;
      if (2 * pr + 1 < M) Brow = Cf + (long)(2 * pr + 1) * d.Nc + row * d.pz;
    }
    b0[line * LP + k] = pair_spectrum<T>(Arow, Brow, k, nz);
  }
  C* res = block_fft<+1, T>(b0, b1, L, LP, pz, tw);
  C* other = (res == b0) ? b1 : b0;
  KahanT<T> psum;  // per-thread partial (a few points); merged in FP64 below
  unsigned st = 0;
  for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
    const int r = e / nz, k = e - r * nz;
    if (row0 + r >= d.rows) continue;
    T nv[11];
#pragma unroll
    for (int a = 0; a < M; ++a) {
      const C z = res[(r * NP + a / 2) * LP + k];
      nv[a] = (a & 1) ? z.y : z.x;
    }
    const T eta = nv[0];
    const T phi = fmt_phi_point<T, MODEL>(nv, ih, ih2, esA, esB);
    if (eta > (T)0.5 && (T)1 - eta < (T)0) st |= 1u;
    if (!isfinite(phi)) st |= 2u;
    psum.add(phi);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const T im = (2 * p + 1 < M) ? nv[2 * p + 1] : (T)0;
      other[(r * NP + p) * LP + k] = mk<T>(nv[2 * p], im);
    }
  }
  if (st) atomicOr(status, st);
  block_kahan_store<1>(&psum, part, blockIdx.x);
  C* res2 = block_fft<-1, T>(other, res, L, LP, pz, tw);
  for (int e = threadIdx.x; e < L * nzc; e += blockDim.x) {
    const int line = e / nzc, k = e - line * nzc;
    const int r = line / NP, pr = line - r * NP;
    const long row = row0 + r;
    if (row >= d.rows) continue;
    const C Z = res2[line * LP + k];
    const C W = res2[line * LP + (k == 0 ? 0 : nz - k)];
    Cf[(long)(2 * pr) * d.Nc + row * d.pz + k] = mk<T>((T)0.5 * (Z.x + W.x), (T)0.5 * (Z.y - W.y));
    if (2 * pr + 1 < M) Cf[(long)(2 * pr + 1) * d.Nc + row * d.pz + k] = mk<T>((T)0.5 * (Z.y + W.y), (T)0.5 * (W.x - Z.x));
  }
}

// ---------------------------------------------------- Hessian z rows ---
// The pointwise step of the Hessian-vector product (FMT::add_second_derivative,
// src/FMT.cpp:437-567): the same row layout as k_phi_rows, with the M fields of
// Cf holding the convolutions of v (z still in spectral form) and NA the M
// weighted densities of the state in real space (M x N). Per point the folded
// (d2Phi).Psi replaces Psi; the rows are transformed back over the inputs.
template <class T, int MODEL>
__global__ void __launch_bounds__(256) k_hess_rows(typename Cx<T>::type* __restrict__ Cf, const T* __restrict__ NA, Dims d, FFTPlan pz,
                                                   const typename Cx<T>::type* __restrict__ tw, int RB, T hsd, T esA, T esB) {
  typedef typename Cx<T>::type C;
  constexpr int M = ModelTraits<MODEL>::M;
  constexpr int NP = (M + 1) / 2;
  const T ih = (T)(1.0 / (double)hsd), ih2 = (T)(1.0 / ((double)hsd * (double)hsd));
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nz = d.nz, LP = nz + 1, nzc = d.nzc;
  const int L = NP * RB;
  C* b0 = reinterpret_cast<C*>(smem_raw);
  C* b1 = b0 + L * LP;
  const long row0 = (long)blockIdx.x * RB;
  for (int e = threadIdx.x; e < L * nz; e += blockDim.x) {
    const int line = e / nz, k = e - line * nz;
    const int r = line / NP, pr = line - r * NP;
    const long row = row0 + r;
    const C* Arow = nullptr;
    const C* Brow = nullptr;
    if (row < d.rows) {
      Arow = Cf + (long)(2 * pr) * d.Nc + row * d.pz;
      if (2 * pr + 1 < M) Brow = Cf + (long)(2 * pr + 1) * d.Nc + row * d.pz;
    }
    b0[line * LP + k] = pair_spectrum<T>(Arow, Brow, k, nz);
  }
  C* res = block_fft<+1, T>(b0, b1, L, LP, pz, tw);
  C* other = (res == b0) ? b1 : b0;
  for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
    const int r = e / nz, k = e - r * nz;
    const long row = row0 + r;
    if (row >= d.rows) continue;
    T nv[11], pv[11];
#pragma unroll
    for (int a = 0; a < M; ++a) {
      const C z = res[(r * NP + a / 2) * LP + k];
      pv[a] = (a & 1) ? z.y : z.x;
      nv[a] = NA[(long)a * d.N + row * nz + k];
    }
    fmt_d2phi_dot_point<T, MODEL>(nv, pv, ih, ih2, esA, esB, ih, ih2);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const T im = (2 * p + 1 < M) ? pv[2 * p + 1] : (T)0;
      other[(r * NP + p) * LP + k] = mk<T>(pv[2 * p], im);
    }
  }
  C* res2 = block_fft<-1, T>(other, res, L, LP, pz, tw);
  for (int e = threadIdx.x; e < L * nzc; e += blockDim.x) {
    const int line = e / nzc, k = e - line * nzc;
    const int r = line / NP, pr = line - r * NP;
    const long row = row0 + r;
    if (row >= d.rows) continue;
    const C Z = res2[line * LP + k];
    const C W = res2[line * LP + (k == 0 ? 0 : nz - k)];
    Cf[(long)(2 * pr) * d.Nc + row * d.pz + k] = mk<T>((T)0.5 * (Z.x + W.x), (T)0.5 * (Z.y - W.y));
    if (2 * pr + 1 < M) Cf[(long)(2 * pr + 1) * d.Nc + row * d.pz + k] = mk<T>((T)0.5 * (Z.y + W.y), (T)0.5 * (W.x - Z.x));
  }
}

// Last step of the Hessian-vector product: c2r of E (FMT + mean-field
// back-convolution of the Lambda fields) and the ideal-gas term,
//   Hv = (v / rho + c2r(E)) dV   (DFT::matrix_dot_v_intern, src/DFT.cpp:455-462).
template <class T, class RT, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256) k_hess_final_rows(const typename Cx<T>::type* __restrict__ E, const double* __restrict__ rho,
                                                         const RT* __restrict__ v, RT* __restrict__ out, Dims d, FFTPlan pz,
                                                         const typename Cx<T>::type* __restrict__ tw, int RB, double dV, int have_fmt_or_mf) {
  typedef typename Cx<T>::type C;
  constexpr bool DS = DfSpectra<T, NF, DFS>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* b0 = reinterpret_cast<C*>(smem_raw);
  const int nz = NF > 0 ? NF : d.nz, LP = nz + 1;
  C* b1 = b0 + RB * LP;
  const long pair0 = (long)blockIdx.x * RB;
  C* res = b0;
  if (have_fmt_or_mf) {
#pragma unroll 4
    for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
      const int r = e / nz, k = e - r * nz;
      const long ra = 2 * (pair0 + r), rb = ra + 1;
      const C* Ar = ra < d.rows ? E + ra * d.pz : nullptr;
      const C* Br = rb < d.rows ? E + rb * d.pz : nullptr;
      if constexpr (DS)
        reinterpret_cast<dfc*>(b0)[r * LP + k] = pair_spectrum_df(reinterpret_cast<const dfc*>(Ar), reinterpret_cast<const dfc*>(Br), k, nz);
      else
        b0[r * LP + k] = pair_spectrum<T>(Ar, Br, k, nz);
    }
    res = rows_fft<+1, T, NF, !DS, !DS>(b0, b1, RB, LP, pz, tw);
  }
  if constexpr (DS) {  // double-float spectra: (v / rho + h) dV in df64, one join per point
    const dfc* rd = reinterpret_cast<const dfc*>(res);
    const dfs dVd = dfs_split(dV);
    for (int e = threadIdx.x; e < 2 * RB * nz; e += blockDim.x) {
      const int rr = e / nz, k = e - rr * nz;
      const long row = 2 * pair0 + rr;
      if (row >= d.rows) continue;
      const long p = row * nz + k;
      dfs h = dfs(0);
      if (have_fmt_or_mf) {
        const dfc z = rd[(rr >> 1) * LP + k];
        h = (rr & 1) ? z.y : z.x;
      }
      const dfs f = (dfs_split((double)v[p]) / dfs_split(rho[p])) * dVd + h * dVd;
      out[p] = (RT)dfs_join(f);
    }
    return;
  }
  const T dVt = (T)dV;
  for (int e = threadIdx.x; e < 2 * RB * nz; e += blockDim.x) {
    const int rr = e / nz, k = e - rr * nz;
    const long row = 2 * pair0 + rr;
    if (row >= d.rows) continue;
    const long p = row * nz + k;
    T h = 0;
    if (have_fmt_or_mf) {
      const C z = res[(rr >> 1) * LP + k];
      h = (rr & 1) ? z.y : z.x;
    }
    const T f = (conv<T>(v[p]) / conv<T>(rho[p])) * dVt + h * dVt;
    out[p] = conv<RT>(f);
  }
}

// ------------------------------------------------------ final z rows ---
// The final row pass's pointwise terms on double-float spectra (FP64 evaluation with
// compile-time plans): ln rho by the table-driven df64 logarithm, every product and sum in
// df64 on the FP32 pipe; rho is split and dF joined once per point, and each thread's sums
// are joined once before the FP64 block merges. Same terms and order as the FP64 loop.
template <class RT>
__device__ __forceinline__ void final_points_df(const double2* __restrict__ res, const RT* __restrict__ rho,
                                                const double* __restrict__ vext, RT* __restrict__ dF, const Dims& d, int RB,
                                                int LP, int nz, long pair0, double dV, double mu, int have_fmt_or_mf, int ideal,
                                                double* __restrict__ part, double* __restrict__ nrm, RT* __restrict__ dF2) {
  const dfc* rd = reinterpret_cast<const dfc*>(res);
  const dfs dVd = dfs_split(dV), mud = dfs_split(mu);
  dfs a0 = dfs(0), a1 = dfs(0), a2 = dfs(0), a3 = dfs(0), aq = dfs(0), mx = dfs(0);
  for (int e = threadIdx.x; e < 2 * RB * nz; e += blockDim.x) {
    const int rr = e / nz, k = e - rr * nz;
    const long row = 2 * pair0 + rr;
    if (row >= d.rows) continue;
    const long p = row * nz + k;
    const dfs r0 = dfs_split((double)rho[p]);
    const dfs lr = df_log(r0);
    dfs f = ideal ? lr * dVd : dfs(0);
    if (have_fmt_or_mf) {
      const dfc z = rd[(rr >> 1) * LP + k];
      f += ((rr & 1) ? z.y : z.x) * dVd;
    }
    dfs ve = dfs(0);
    if (vext) {
      ve = dfs_split(vext[p]);
      f += ve * dVd;
    }
    f += -mud * dVd;
    const RT fv = (RT)dfs_join(f);
    dF[p] = fv;
    if (dF2) dF2[p] = fv;
    if (ideal) a0 += (r0 * lr - r0) * dVd;
    a1 += r0;
    if (vext) a2 += ve * r0;
    a3 += f * r0;
    if (nrm) {
      aq += f * f;
      const dfs af = df_abs(f);
      if (mx < af) mx = af;
    }
  }
  KahanT<double> ks[4];
  ks[0].add(dfs_join(a0));
  ks[1].add(dfs_join(a1));
  ks[2].add(dfs_join(a2));
  ks[3].add(dfs_join(a3));
  block_kahan_store<4>(ks, part, blockIdx.x);
  if (nrm) {
    KahanT<double> kq;
    kq.add(dfs_join(aq));
    block_norms_store<double>(kq, dfs_join(mx), nrm, blockIdx.x);
  }
}

// c2r of E (the summed hard-sphere + mean-field back-convolution) and the
// pointwise terms of DFT::calculateFreeEnergyAndDerivatives_internal_
// (src/DFT.cpp:377-425) and Species::externalField (src/Species.cpp:51-61):
//   dF = ln(rho) dV + c2r(E) dV + V_ext dV - mu dV
// with FP64 partial sums: F_id = sum (rho ln rho - rho) dV, sum rho,
// sum V_ext rho, sum dF rho (for the fixed-mass projection).
template <class T, class RT = double, int NF = 0, bool DFS = false>
__global__ void __launch_bounds__(256) k_final_rows(const typename Cx<T>::type* __restrict__ E, const RT* __restrict__ rho,
                                                    const double* __restrict__ vext, RT* __restrict__ dF, Dims d, FFTPlan pz,
                                                    const typename Cx<T>::type* __restrict__ tw, int RB, double dV, double mu,
                                                    int have_fmt_or_mf, int ideal, double* __restrict__ part,
                                                    double* __restrict__ nrm, RT* __restrict__ dF2 = nullptr) {
  typedef typename Cx<T>::type C;
  constexpr bool DS = DfSpectra<T, NF, DFS>::value;
  if constexpr (DS) {
    df_log_table_init(threadIdx.x, blockDim.x);
    __syncthreads();
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* b0 = reinterpret_cast<C*>(smem_raw);
  const int nz = NF > 0 ? NF : d.nz, LP = nz + 1;
  C* b1 = b0 + RB * LP;
  const long pair0 = (long)blockIdx.x * RB;
  {  // the block's densities (its rows are consecutive) into L2 now: they are read after the
     // transform, and by then the evaluation's earlier passes have long evicted them
    const char* r0 = reinterpret_cast<const char*>(rho + 2 * pair0 * nz);
    const long nbytes = (long)(min(2L * RB, d.rows - 2 * pair0) * nz) * (long)sizeof(RT);
    for (long o = (long)threadIdx.x * 128; o < nbytes; o += (long)blockDim.x * 128)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(r0 + o));
  }
  C* res = b0;
  if (have_fmt_or_mf) {
#pragma unroll 4
    for (int e = threadIdx.x; e < RB * nz; e += blockDim.x) {
      const int r = e / nz, k = e - r * nz;
      const long ra = 2 * (pair0 + r), rb = ra + 1;
      const C* Ar = ra < d.rows ? E + ra * d.pz : nullptr;
      const C* Br = rb < d.rows ? E + rb * d.pz : nullptr;
      if constexpr (DS)
        reinterpret_cast<dfc*>(b0)[r * LP + k] = pair_spectrum_df(reinterpret_cast<const dfc*>(Ar), reinterpret_cast<const dfc*>(Br), k, nz);
      else
        b0[r * LP + k] = pair_spectrum<T>(Ar, Br, k, nz);
    }
    res = rows_fft<+1, T, NF, !DS, !DS>(b0, b1, RB, LP, pz, tw);
  }
  if constexpr (DS) {  // double-float spectra: the pointwise terms in df64 too
    final_points_df(res, rho, vext, dF, d, RB, LP, nz, pair0, dV, mu, have_fmt_or_mf, ideal, part, nrm, dF2);
    return;
  }
  // Pointwise terms in the bulk precision T (FP64 in FP64 mode); each thread
  // keeps Kahan partials in T over its few points, merged in FP64 across the
  // block and with compensation across blocks.
  KahanT<T> ks[4];
  KahanT<T> kq;  // sum of dF^2 and max |dF| when nrm is set (the residual norms, fused here)
  T mx = 0;
  const T dVt = (T)dV, mut = (T)mu;
  for (int e = threadIdx.x; e < 2 * RB * nz; e += blockDim.x) {
    const int rr = e / nz, k = e - rr * nz;
    const long row = 2 * pair0 + rr;
    if (row >= d.rows) continue;
    const long p = row * nz + k;
    const T r0 = conv<T>(rho[p]);
    const T lr = ln_t<T>(r0);
    T h = 0;
    if (have_fmt_or_mf) {
      const C z = res[(rr >> 1) * LP + k];
      h = (rr & 1) ? z.y : z.x;
    }
    const T ve = vext ? (T)vext[p] : (T)0;
    T f = ideal ? lr * dVt : (T)0;
    f += h * dVt;
    f += ve * dVt;
    f += -mut * dVt;
    dF[p] = conv<RT>(f);
    if (dF2) dF2[p] = conv<RT>(f);
    if (ideal) ks[0].add((r0 * lr - r0) * dVt);
    ks[1].add(r0);
    ks[2].add(ve * r0);
    ks[3].add(f * r0);
    if (nrm) {
      kq.add(f * f);
      const T af = f < (T)0 ? -f : f;
      mx = af > mx ? af : mx;
    }
  }
  block_kahan_store<4>(ks, part, blockIdx.x);
  if (nrm) block_norms_store<T>(kq, mx, nrm, blockIdx.x);
}

// ----------------------------------------------------------- pointwise ---
__global__ void k_scale(double* __restrict__ x, long n, const double* __restrict__ num, double den_scale, double target);
__global__ void k_add_scalar(double* __restrict__ x, long n, const double* __restrict__ v, double scale);

}  // namespace cdft

// Shared-memory FFT building blocks for sm_103a.
//
// A thread block transforms L lines of length n held in shared memory with a
// mixed-radix Stockham (self-sorting) decimation-in-frequency scheme: at a
// stage of radix p on sub-length len (stride s, m = len/p)
//     y[k + s*(p*q + t)] = (sum_j x[k + s*(q + m*j)] w_p^{jt}) * w_len^{qt}
// for q < m, k < s. Twiddles come from a per-length table built on the host in
// long double (exp(-2 pi i q t / len) per stage, plus the p-th roots), so FP64
// transforms keep ~1 ulp twiddle accuracy. Radices: 8, 4, 2, 3, 5, 7, and a
// generic direct DFT for any other prime up to 31.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "cdft_types.h"

namespace cdft {

template <class T> __host__ __device__ __forceinline__ typename Cx<T>::type mk(T a, T b) {
  typename Cx<T>::type r; r.x = a; r.y = b; return r;
}
template <class C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <class C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// multiply by conj(b) when DIR > 0 (backward), by b when DIR < 0 (forward)
template <int DIR, class C> __device__ __forceinline__ C cmul_dir(C a, C b) {
  if (DIR < 0) return cmul(a, b);
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
// multiply by -i (forward) or +i (backward)
template <int DIR, class C> __device__ __forceinline__ C cmul_mi(C a) {
  C r;
  if (DIR < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
  return r;
}
template <class C, class T> __device__ __forceinline__ C cscale(C a, T s) { a.x *= s; a.y *= s; return a; }

template <int DIR, class C>
__device__ __forceinline__ void dft2(C* a) {
  C t = a[0]; a[0] = cadd(t, a[1]); a[1] = csub(t, a[1]);
}
template <int DIR, class C>
__device__ __forceinline__ void dft4(C* a) {
  C t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]), t2 = cadd(a[1], a[3]), t3 = cmul_mi<DIR>(csub(a[1], a[3]));
  a[0] = cadd(t0, t2); a[2] = csub(t0, t2); a[1] = cadd(t1, t3); a[3] = csub(t1, t3);
}
template <int DIR, class T, class C>
__device__ __forceinline__ void dft8(C* a) {
  const T r = (T)0.70710678118654752440084436210484903928;
  C e[4] = {a[0], a[2], a[4], a[6]}, o[4] = {a[1], a[3], a[5], a[7]};
  dft4<DIR>(e);
  dft4<DIR>(o);
  // twiddles w8^k for k = 1, 2, 3 applied to the odd half
  C o1 = o[1], o3 = o[3];
  if (DIR < 0) {
    o[1] = mk<T>(r * (o1.x + o1.y), r * (o1.y - o1.x));
    o[3] = mk<T>(r * (o3.y - o3.x), -r * (o3.x + o3.y));
  } else {
    o[1] = mk<T>(r * (o1.x - o1.y), r * (o1.x + o1.y));
    o[3] = mk<T>(-r * (o3.x + o3.y), r * (o3.x - o3.y));
  }
  o[2] = cmul_mi<DIR>(o[2]);
  for (int k = 0; k < 4; ++k) { a[k] = cadd(e[k], o[k]); a[k + 4] = csub(e[k], o[k]); }
}

// One radix-P butterfly of a Stockham stage: loads x[k + s*(q + m*j)],
// applies the P-point DFT and the stage twiddles, stores y[k + s*(P*q + t)].
// UNIT: every stage twiddle is 1 (the last stage, m = 1): no products with them.
template <int DIR, class T, int P, bool UNIT = false>
__device__ __forceinline__ void butterfly(const typename Cx<T>::type* __restrict__ xl, typename Cx<T>::type* __restrict__ yl,
                                          int q, int k, int m, int s, const typename Cx<T>::type* __restrict__ tw,
                                          const typename Cx<T>::type* __restrict__ roots) {
  typedef typename Cx<T>::type C;
  C a[P];
#pragma unroll
  for (int j = 0; j < P; ++j) a[j] = xl[k + s * (q + m * j)];
  if (P == 8) {
    dft8<DIR, T>(a);
  } else if (P == 4) {
    dft4<DIR>(a);
  } else if (P == 2) {
    dft2<DIR>(a);
  } else {
    C w[P];
#pragma unroll
    for (int j = 0; j < P; ++j) w[j] = __ldg(reinterpret_cast<const C*>(roots + j));
    C b[P];
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
  yl[k + s * (P * q)] = a[0];
#pragma unroll
  for (int t = 1; t < P; ++t) {
    if constexpr (UNIT) yl[k + s * (P * q + t)] = a[t];
    else yl[k + s * (P * q + t)] = cmul_dir<DIR>(a[t], __ldg(reinterpret_cast<const C*>(twq + t)));
  }
}

// Any other prime radix (up to kMaxRadix): direct DFT through local memory.
template <int DIR, class T>
__device__ void butterfly_generic(const typename Cx<T>::type* __restrict__ xl, typename Cx<T>::type* __restrict__ yl, int q,
                                  int k, int m, int s, int p, const typename Cx<T>::type* __restrict__ tw,
                                  const typename Cx<T>::type* __restrict__ roots) {
  typedef typename Cx<T>::type C;
  C in[kMaxRadix];
  for (int j = 0; j < p; ++j) in[j] = xl[k + s * (q + m * j)];
  const C* twq = tw + q * p;
  for (int t = 0; t < p; ++t) {
    C acc = in[0];
    int idx = 0;
    for (int j = 1; j < p; ++j) {
      idx += t;
      if (idx >= p) idx -= p;
      acc = cadd(acc, cmul_dir<DIR>(in[j], roots[idx]));
    }
    yl[k + s * (p * q + t)] = (t == 0) ? acc : cmul_dir<DIR>(acc, twq[t]);
  }
}

// One Stockham stage over L lines (pitch LP elements) in shared memory.
template <int DIR, class T>
__device__ __forceinline__ void fft_stage(const typename Cx<T>::type* __restrict__ x, typename Cx<T>::type* __restrict__ y,
                                          int L, int LP, int len, int s, int p, const typename Cx<T>::type* __restrict__ tw,
                                          const typename Cx<T>::type* __restrict__ roots) {
  const int m = len / p;
  const int per_line = m * s;
  const int total = L * per_line;
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    const int line = w / per_line;
    const int u = w - line * per_line;
    const int q = u / s, k = u - q * s;
    const typename Cx<T>::type* xl = x + line * LP;
    typename Cx<T>::type* yl = y + line * LP;
    switch (p) {
      case 8: butterfly<DIR, T, 8>(xl, yl, q, k, m, s, tw, roots); break;
      case 4: butterfly<DIR, T, 4>(xl, yl, q, k, m, s, tw, roots); break;
      case 2: butterfly<DIR, T, 2>(xl, yl, q, k, m, s, tw, roots); break;
      case 3: butterfly<DIR, T, 3>(xl, yl, q, k, m, s, tw, roots); break;
      case 5: butterfly<DIR, T, 5>(xl, yl, q, k, m, s, tw, roots); break;
      case 7: butterfly<DIR, T, 7>(xl, yl, q, k, m, s, tw, roots); break;
      default: butterfly_generic<DIR, T>(xl, yl, q, k, m, s, p, tw, roots); break;
    }
  }
}

// Transforms L lines held in buf0 (pitch LP); buf1 is scratch of the same size.
// Returns the buffer that holds the result. Ends with __syncthreads().
template <int DIR, class T>
__device__ typename Cx<T>::type* block_fft(typename Cx<T>::type* buf0, typename Cx<T>::type* buf1, int L, int LP,
                                           const FFTPlan& P, const typename Cx<T>::type* __restrict__ table) {
  typedef typename Cx<T>::type C;
  C* src = buf0;
  C* dst = buf1;
  int len = P.n, s = 1;
  for (int st = 0; st < P.nst; ++st) {
    const int p = P.radix[st];
    __syncthreads();
    fft_stage<DIR, T>(src, dst, L, LP, len, s, p, table + P.tw_off[st], table + P.root_off[st]);
    C* t = src; src = dst; dst = t;
    len /= p;
    s *= p;
  }
  __syncthreads();
  return src;
}

// The same transform with the plan of length NF resolved at compile time (the
// default radix order of make_fft_table; radix_at / len_at / twoff_at restate
// that order as constant expressions).
__host__ __device__ constexpr int radix_at(int n, int i) {
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
__host__ __device__ constexpr int len_at(int n, int i) {
  int len = n;
  for (int st = 0; st < i; ++st) len /= radix_at(n, st);
  return len;
}
__host__ __device__ constexpr int twoff_at(int n, int i) {
  int off = 0, len = n;
  for (int st = 0; st < i; ++st) {
    const int p = radix_at(n, st);
    off += len + p;
    len /= p;
  }
  return off;
}

template <int DIR, class T, int NF, int ST = 0>
__device__ __forceinline__ typename Cx<T>::type* block_fft_fixed(typename Cx<T>::type* src, typename Cx<T>::type* dst, int L, int LP,
                                                                 const typename Cx<T>::type* __restrict__ table) {
  typedef typename Cx<T>::type C;
  __syncthreads();
  if constexpr (radix_at(NF, ST) == 0) {
    return src;
  } else {
    constexpr int p = radix_at(NF, ST), len = len_at(NF, ST), m = len / p, s = NF / len, per_line = m * s;
    const C* tw = table + twoff_at(NF, ST);
    const C* rt = tw + len;
    const int total = L * per_line;
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
      const int line = w / per_line, u = w - line * per_line;
      const int q = u / s, k = u - q * s;
      const C* xl = src + line * LP;
      C* yl = dst + line * LP;
      if constexpr (p == 2 || p == 3 || p == 4 || p == 5 || p == 7 || p == 8) butterfly<DIR, T, p, m == 1>(xl, yl, q, k, m, s, tw, rt);
      else butterfly_generic<DIR, T>(xl, yl, q, k, m, s, p, tw, rt);
    }
    return block_fft_fixed<DIR, T, NF, ST + 1>(dst, src, L, LP, table);
  }
}

// Runtime plan when NF == 0, the compile-time plan of length NF otherwise.
template <int DIR, class T, int NF>
__device__ __forceinline__ typename Cx<T>::type* block_fft_nf(typename Cx<T>::type* b0, typename Cx<T>::type* b1, int L, int LP,
                                                              const FFTPlan& P, const typename Cx<T>::type* __restrict__ table) {
  if constexpr (NF > 0) {
    typename Cx<T>::type* r = block_fft_fixed<DIR, T, NF>(b0, b1, L, LP, table);
    __syncthreads();
    return r;
  } else {
    return block_fft<DIR, T>(b0, b1, L, LP, P, table);
  }
}

}  // namespace cdft

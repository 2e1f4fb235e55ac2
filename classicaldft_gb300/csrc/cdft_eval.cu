// Evaluation engine: FFT tables, weight spectra, and the launch sequence of
// one F+dF evaluation (kernels in cdft_kernels.cuh).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include "cdft_internal.h"
#include "cdft_kernels.cuh"
#include "cdft_kernels_tma.cuh"
#include "cdft_phi_launch.h"

namespace cdft {

#define CK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) {                                                                    \
      if (err) *err = std::string(#x) + ": " + cudaGetErrorString(e_);                          \
      return 5;                                                                                 \
    }                                                                                           \
  } while (0)

// ------------------------------------------------------------ FFT tables ---
FFTTable::~FFTTable() {
  if (d64) cudaFree(d64);
  if (d32) cudaFree(d32);
}

// Calls f(std::integral_constant<int, NF>) with the compile-time plan length NF
// of an axis (128, 256, or 0 for the runtime plan): the kernels are instantiated
// once per length.
template <class F>
inline void with_nf(int nf, F&& f) {
  if (nf == 128) f(std::integral_constant<int, 128>());
  else if (nf == 256) f(std::integral_constant<int, 256>());
  else f(std::integral_constant<int, 0>());
}

// with_nf, and whether the launch's spectra are double-float (f's second argument,
// std::true_type only for FP64 with a compile-time plan and io set)
template <class T, class F>
inline void with_nf_io(int nf, bool io, F&& f) {
  with_nf(nf, [&](auto nf_) {
    constexpr int NF = decltype(nf_)::value;
    if constexpr (kDf64Transforms && std::is_same<T, double>::value && NF > 0) {
      if (io) f(nf_, std::true_type());
      else f(nf_, std::false_type());
    } else {
      f(nf_, std::false_type());
    }
  });
}

std::vector<int> default_radices(int n) {
  std::vector<int> r;
  int m = n;
  while (m > 1) {
    int f = 0;
    if (m % 8 == 0 && m != 16) f = 8;  // 16 = 4 x 4 keeps both stages radix 4
    else if (m % 4 == 0) f = 4;
    else if (m % 2 == 0) f = 2;
    else {
      for (int q = 3; q <= m; q += 2)
        if (m % q == 0) { f = q; break; }
    }
    r.push_back(f);
    m /= f;
  }
  return r;
}

std::shared_ptr<FFTTable> make_fft_table(int n, std::string* err, const std::vector<int>* radices) {
  auto t = std::make_shared<FFTTable>();
  FFTPlan& P = t->plan;
  std::memset(&P, 0, sizeof(P));
  P.n = n;
  const std::vector<int> rad = radices ? *radices : default_radices(n);
  long prod = 1;
  for (int r : rad) {
    if (r < 2 || r > kMaxRadix || P.nst >= kMaxStages) {
      if (err) *err = "grid length " + std::to_string(n) + " has a prime factor above 31";
      return nullptr;
    }
    P.radix[P.nst++] = r;
    prod *= r;
  }
  if (prod != n) {
    if (err) *err = "radix ordering does not multiply to " + std::to_string(n);
    return nullptr;
  }
  // table: for each stage the m*p twiddles exp(-2 pi i q t/len), then the p roots exp(-2 pi i t/p)
  std::vector<long double> re, im;
  auto push = [&](long num, long den) {
    num %= den;
    const long double a = 6.283185307179586476925286766559005768L * (long double)num / (long double)den;
    re.push_back(cosl(a));
    im.push_back(-sinl(a));
  };
  int len = n;
  for (int st = 0; st < P.nst; ++st) {
    const int p = P.radix[st], sub = len / p;
    P.tw_off[st] = (int)re.size();
    for (int q = 0; q < sub; ++q)
      for (int tt = 0; tt < p; ++tt) push((long)q * tt, len);
    P.root_off[st] = (int)re.size();
    for (int tt = 0; tt < p; ++tt) push(tt, p);
    len = sub;
  }
  const size_t cnt = re.size();
  // the FP64 table, then, for the compile-time lengths, the twiddles of the df64
  // transforms' radix order (fxd_radix) as df64 pairs (hi, lo of the real part, hi, lo of
  // the imaginary part), in the same entry layout
  std::vector<long double> dre, dim;
  if (n == 128 || n == 256) {
    int dlen = n;
    for (int st = 0; fxd_radix(n, st) != 0; ++st) {
      const int p = fxd_radix(n, st), sub = dlen / p;
      for (int q = 0; q < sub; ++q)
        for (int tt = 0; tt < p; ++tt) {
          const long double a = 6.283185307179586476925286766559005768L * (long double)(((long)q * tt) % dlen) / (long double)dlen;
          dre.push_back(cosl(a));
          dim.push_back(-sinl(a));
        }
      for (int tt = 0; tt < p; ++tt) {
        const long double a = 6.283185307179586476925286766559005768L * (long double)tt / (long double)p;
        dre.push_back(cosl(a));
        dim.push_back(-sinl(a));
      }
      dlen = sub;
    }
  }
  const size_t dcnt = dre.size();
  std::vector<double2> h64(cnt + dcnt);
  std::vector<float2> h32(cnt);
  for (size_t i = 0; i < cnt; ++i) {
    h64[i] = make_double2((double)re[i], (double)im[i]);
    h32[i] = make_float2((float)re[i], (float)im[i]);
  }
  for (size_t i = 0; i < dcnt; ++i) {
    const float rh = (float)dre[i], ih = (float)dim[i];
    const float rl = (float)(dre[i] - (long double)rh), il = (float)(dim[i] - (long double)ih);
    float4 q = make_float4(rh, rl, ih, il);
    std::memcpy(&h64[cnt + i], &q, sizeof(q));
  }
  if (cudaMalloc(&t->d64, (cnt + dcnt) * sizeof(double2)) != cudaSuccess || cudaMalloc(&t->d32, cnt * sizeof(float2)) != cudaSuccess) {
    if (err) *err = "cudaMalloc of FFT tables failed";
    return nullptr;
  }
  cudaMemcpy(t->d64, h64.data(), (cnt + dcnt) * sizeof(double2), cudaMemcpyHostToDevice);
  cudaMemcpy(t->d32, h32.data(), cnt * sizeof(float2), cudaMemcpyHostToDevice);
  return t;
}

template <class T> const typename Cx<T>::type* twp(const FFTTable* t);
template <> const double2* twp<double>(const FFTTable* t) { return reinterpret_cast<const double2*>(t->d64); }
template <> const float2* twp<float>(const FFTTable* t) { return reinterpret_cast<const float2*>(t->d32); }

// --------------------------------------------------------- small kernels ---
__global__ void k_finish_reduce(const double* __restrict__ part, long nblk, int nv, double* __restrict__ out) {
  // one block; thread t sums blocks t, t+256, ... in order; then a fixed tree
  __shared__ double ss[256], sc[256];
  for (int v = 0; v < nv; ++v) {
    Acc a;
    a.init();
    for (long b = threadIdx.x; b < nblk; b += blockDim.x) a.merge(part[(b * nv + v) * 2], part[(b * nv + v) * 2 + 1]);
    ss[threadIdx.x] = a.s;
    sc[threadIdx.x] = a.c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) {
        Acc t;
        t.s = ss[threadIdx.x];
        t.c = sc[threadIdx.x];
        t.merge(ss[threadIdx.x + o], sc[threadIdx.x + o]);
        ss[threadIdx.x] = t.s;
        sc[threadIdx.x] = t.c;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[v] = ss[0] + sc[0];
    __syncthreads();
  }
}

// All sums of one evaluation in one launch: warp w finishes sum w of the three
// partial-sum segments (Phi: 1 value, mean field: 1, final rows: 4) — each lane
// merges blocks lane, lane + 32, ... in order, then a fixed shuffle tree. Short,
// independent FP64 chains per warp instead of three single-block kernels.
struct FinishSeg {
  const double* part;
  long nblk;
  int nv;
  double* out;
};
__global__ void __launch_bounds__(224) k_finish_terms(FinishSeg s0, FinishSeg s1, FinishSeg s2, FinishSeg s3) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const FinishSeg* segs[4] = {&s0, &s1, &s2, &s3};
  int v = w;
  const FinishSeg* sg = nullptr;
  for (int i = 0; i < 4; ++i) {
    if (segs[i]->nv <= 0 || !segs[i]->part) continue;
    if (v < segs[i]->nv) { sg = segs[i]; break; }
    v -= segs[i]->nv;
  }
  if (!sg) return;
  Acc a;
  a.init();
  for (long b = lane; b < sg->nblk; b += 32) a.merge(sg->part[(b * sg->nv + v) * 2], sg->part[(b * sg->nv + v) * 2 + 1]);
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_down_sync(0xffffffffu, a.s, o), c2 = __shfl_down_sync(0xffffffffu, a.c, o);
    if (lane < o) a.merge(s2, c2);
  }
  if (lane == 0) sg->out[v] = a.s + a.c;
}

template <class T>
__global__ void k_compact(const double2* __restrict__ full, T* __restrict__ out, long n, int odd, double scale) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = (T)((odd ? full[i].y : full[i].x) * scale);
}
// FP64 values to df64 pairs (hi = RN(d), lo = RN(d - hi))
__global__ void k_split_df(const double* __restrict__ in, float2* __restrict__ out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const dfs v = dfs_split(in[i]);
    out[i] = make_float2(v.h, v.l);
  }
}
template <class T>
__global__ void k_round_spectra(const double* __restrict__ in, T* __restrict__ out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) out[i] = (T)in[i];
}

// ------------------------------------------------------------------ AO ---
// FMT_AO_Species (src/FMT_Species.cpp:694-738, include/Species.h:428-443, src/FMT.cpp:393-421).
// Psi~ = sum_a w~p_a S_a: the polymer weights times the spectra of the polymer-folded
// derivative fields (FMT_Weighted_Density::add_weight_schur_dPhi_to_arg: no conjugate, the
// vector parity is in the fields' sign).
template <class T>
__global__ void k_ao_psi(const typename Cx<T>::type* __restrict__ S, const T* __restrict__ w, int M, long Nc,
                         typename Cx<T>::type* __restrict__ psi) {
  typedef typename Cx<T>::type C;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < Nc; i += (long)gridDim.x * blockDim.x) {
    C acc = mk<T>(0, 0);
    for (int a = 0; a < M; ++a) acc = cadd(acc, mul_weight(S[(long)a * Nc + i], w[(long)a * Nc + i], weight_is_odd(a)));
    psi[i] = acc;
  }
}
// x <- exp(-x) in place, with the block partials of sum exp(-x) (the AO free energy)
template <class T>
__global__ void __launch_bounds__(256) k_ao_exp(T* __restrict__ x, long n, double* __restrict__ part) {
  KahanT<T> acc;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const T e = exp_t<T>(-x[i]);
    x[i] = e;
    acc.add(e);
  }
  block_kahan_store<1>(&acc, part, blockIdx.x);
}
// Upsilon~_a = w~p_a e~ (FMT_Weighted_Density::convoluteWith of exp(-Psi) with the polymer weights)
template <class T>
__global__ void k_ao_upsilon(const typename Cx<T>::type* __restrict__ e, const T* __restrict__ w, int M, long Nc,
                             typename Cx<T>::type* __restrict__ S) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < Nc; i += (long)gridDim.x * blockDim.x) {
    const typename Cx<T>::type z = e[i];
    for (int a = 0; a < M; ++a) S[(long)a * Nc + i] = mul_weight(z, w[(long)a * Nc + i], weight_is_odd(a));
  }
}
// per point: X_a <- reservoir * [sum_b d2Phi(n)/dn_a dn_b Upsilon_b] folded with the colloid
// diameter, Upsilon read with the polymer diameter (FMT::calculateFreeEnergyAndDerivatives'
// AO part, src/FMT.cpp:393-421); the reference's later x reservoir x dV is folded here and in
// the final row pass's dV.
template <class T, int MODEL>
__global__ void __launch_bounds__(256) k_ao_force(const T* __restrict__ NA, T* __restrict__ X, long N, T ih, T ih2, T A, T B, T iph,
                                                  T iph2, T res) {
  constexpr int M = ModelTraits<MODEL>::M;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < N; p += (long)gridDim.x * blockDim.x) {
    T nd[11], up[11];
#pragma unroll
    for (int a = 0; a < 11; ++a) {
      nd[a] = a < M ? NA[(long)a * N + p] : (T)0;
      up[a] = a < M ? X[(long)a * N + p] : (T)0;
    }
    fmt_d2phi_dot_point<T, MODEL>(nd, up, ih, ih2, A, B, iph, iph2);
    if (ModelTraits<MODEL>::tensor) {
      // The reference stores the result's tensor through setFundamentalMeasures_AO
      // (include/Species.h:406-426), whose writes of (j, k) and (k, j) land in the same
      // symmetric slot, the second overwriting the first: an off-diagonal slot carries one
      // of the two equal entries, where the folded form above sums both. Kept as the
      // reference computes it.
      up[6] *= (T)0.5;
      up[7] *= (T)0.5;
      up[9] *= (T)0.5;
    }
#pragma unroll
    for (int a = 0; a < M; ++a) X[(long)a * N + p] = res * up[a];
  }
}
template <class T>
__global__ void k_spec_add(typename Cx<T>::type* __restrict__ dst, const typename Cx<T>::type* __restrict__ src, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) dst[i] = cadd(dst[i], src[i]);
}

// ------------------------------------------------------------ Evaluator ---
template <class T>
Evaluator<T>::~Evaluator() {
  cudaFree(A_); cudaFree(Cf_); cudaFree(E_); cudaFree(w_); cudaFree(watt_); cudaFree(part_); cudaFree(terms_); cudaFree(status_);
  cudaFree(NA_);
  cudaFree(wao_); cudaFree(XA_); cudaFree(S_); cudaFree(psi_); cudaFree(psir_); cudaFree(part_ao_);
  cudaFree(wdf_); cudaFree(wattdf_);
}

template <class T>
long Evaluator<T>::grid_blocks_rows() const {
  const long pairs = (rows_ + 1) / 2;
  return (pairs + rb_rows_ - 1) / rb_rows_;
}

static size_t smem_bytes(int lines, int n, size_t csize, int nbuf) { return (size_t)nbuf * lines * (n + 1) * csize; }

// The dynamic shared-memory limit is an attribute of the kernel, shared by
// every context in the process: raise it to what this context needs, never
// lower it below what another context (another grid) already launches with.
template <class F>
static void raise_smem(F f, size_t bytes) {
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, f) == cudaSuccess && (size_t)a.maxDynamicSharedSizeBytes >= bytes) return;
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <class T, class F>
static void set_smem(F f, size_t bytes) {
  raise_smem(f, bytes);
}

// FP64 real -> full FP64 half spectrum with the double-precision kernels.
static void r2c_f64(const double* in, double2* out, const Dims& d, FFTTable* tx, FFTTable* ty, FFTTable* tz, cudaStream_t s) {
  const int RB = 16, TC = 16;
  const long pairs = (d.rows + 1) / 2;
  const size_t sm_r = smem_bytes(RB, d.nz, sizeof(double2), 2);
  set_smem<double>(k_rows_r2c<double, double>, sm_r);
  k_rows_r2c<double, double><<<(unsigned)((pairs + RB - 1) / RB), 256, sm_r, s>>>(in, out, d, tz->plan, twp<double>(tz), RB);
  const size_t sm_y = smem_bytes(TC, d.ny, sizeof(double2), 2);
  set_smem<double>(k_cols_fft<double, -1>, sm_y);
  k_cols_fft<double, -1><<<dim3((unsigned)(((long)d.nx * d.nzc + TC - 1) / TC), 1), 256, sm_y, s>>>(out, 0, 1, d, ty->plan, twp<double>(ty), TC);
  const size_t sm_x = smem_bytes(TC, d.nx, sizeof(double2), 2);
  set_smem<double>(k_cols_fft<double, -1>, std::max(sm_x, sm_y));
  k_cols_fft<double, -1><<<dim3((unsigned)(((long)d.ny * d.pz + TC - 1) / TC), 1), 256, sm_x, s>>>(out, 0, 0, d, tx->plan, twp<double>(tx), TC);
}


// ------------------------------------------------------- tensor maps ---
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                   const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// rank-dimensional map over 4- or 8-byte elements; dims[0] innermost, strides in bytes for dims 1..rank-1.
static bool encode_map(CUtensorMap* m, int elem_bytes, void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                       const uint32_t* box) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t gd[5], gs[4];
  cuuint32_t bx[5], es[5];
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = box[i];
    es[i] = 1;
    if (i > 0) gs[i - 1] = strides[i - 1];
  }
  const CUtensorMapDataType t = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return fn(m, t, (cuuint32_t)rank, base, gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class T>
bool Evaluator<T>::setup_tma(std::string* err) {
  (void)err;
  constexpr int TC = TileCols<T>::value, E = ElemsPerComplex<T>::value;
  if (nx_ > 256 || ny_ > 256 || nx_ < 8 || ny_ < 8) return false;
  const uint64_t ncol = (uint64_t)ny_ * pz_;  // x-pass columns
  const uint64_t cb = sizeof(C);              // complex bytes
  bool ok = true;
  {  // x-pass maps: {ncol*E, nx, fields}
    uint64_t dims[3] = {ncol * E, (uint64_t)nx_, 1};
    uint64_t str[2] = {ncol * cb, (uint64_t)Nc_ * cb};
    uint32_t box[3] = {(uint32_t)(TC * E), (uint32_t)nx_, 1};
    ok = ok && encode_map(&mapA_, 8, A_, 3, dims, str, box);
    ok = ok && encode_map(&mapE_, 8, E_, 3, dims, str, box);
    if (M_ > 0) {
      dims[2] = (uint64_t)M_;
      ok = ok && encode_map(&mapCf_, 8, Cf_, 3, dims, str, box);
      uint64_t wd[3] = {ncol, (uint64_t)nx_, (uint64_t)M_};
      uint64_t ws[2] = {ncol * sizeof(T), (uint64_t)Nc_ * sizeof(T)};
      uint32_t wb[3] = {(uint32_t)TC, (uint32_t)nx_, 1};
      ok = ok && encode_map(&mapW_, (int)sizeof(T), w_, 3, wd, ws, wb);
    }
    if (mf_) {
      uint64_t wd[3] = {ncol, (uint64_t)nx_, 1};
      uint64_t ws[2] = {ncol * sizeof(T), (uint64_t)Nc_ * sizeof(T)};
      uint32_t wb[3] = {(uint32_t)TC, (uint32_t)nx_, 1};
      ok = ok && encode_map(&mapWatt_, (int)sizeof(T), watt_, 3, wd, ws, wb);
    }
    // FP64 with compile-time plans on every axis: df64 copies of the weights for the
    // double-float-spectra x passes (same geometry, 8-byte elements)
    if (std::is_same<T, double>::value && fx_ > 0 && fy_ > 0 && fz_ > 0) {
      const unsigned cg = (unsigned)std::min<long>(((long)std::max(M_, 1) * Nc_ + 255) / 256, 4096);
      if (M_ > 0) {
        if (!wdf_ && cudaMalloc(&wdf_, (size_t)M_ * Nc_ * sizeof(float2)) != cudaSuccess) return false;
        k_split_df<<<cg, 256>>>(reinterpret_cast<const double*>(w_), static_cast<float2*>(wdf_), (long)M_ * Nc_);
        uint64_t wd[3] = {ncol, (uint64_t)nx_, (uint64_t)M_};
        uint64_t ws[2] = {ncol * 8, (uint64_t)Nc_ * 8};
        uint32_t wb[3] = {(uint32_t)TC, (uint32_t)nx_, 1};
        ok = ok && encode_map(&mapWdf_, 8, wdf_, 3, wd, ws, wb);
      }
      if (mf_) {
        if (!wattdf_ && cudaMalloc(&wattdf_, (size_t)Nc_ * sizeof(float2)) != cudaSuccess) return false;
        k_split_df<<<cg, 256>>>(reinterpret_cast<const double*>(watt_), static_cast<float2*>(wattdf_), Nc_);
        uint64_t wd[3] = {ncol, (uint64_t)nx_, 1};
        uint64_t ws[2] = {ncol * 8, (uint64_t)Nc_ * 8};
        uint32_t wb[3] = {(uint32_t)TC, (uint32_t)nx_, 1};
        ok = ok && encode_map(&mapWattdf_, 8, wattdf_, 3, wd, ws, wb);
      }
      if (cudaDeviceSynchronize() != cudaSuccess) return false;
    }
  }
  constexpr int TCY = TileColsY<T>::value;
  {  // y-pass maps: {pz*E, ny, nx, fields}
    uint64_t dims[4] = {(uint64_t)pz_ * E, (uint64_t)ny_, (uint64_t)nx_, 1};
    uint64_t str[3] = {(uint64_t)pz_ * cb, (uint64_t)ny_ * pz_ * cb, (uint64_t)Nc_ * cb};
    uint32_t box[4] = {(uint32_t)(TCY * E), (uint32_t)ny_, 1, 1};
    ok = ok && encode_map(&mapYA_, 8, A_, 4, dims, str, box);
    ok = ok && encode_map(&mapYE_, 8, E_, 4, dims, str, box);
    if (M_ > 0) {
      dims[3] = (uint64_t)M_;
      ok = ok && encode_map(&mapYC_, 8, Cf_, 4, dims, str, box);
    }
  }
  if (!ok) return false;
  const size_t tile_x = r128((size_t)nx_ * TC * sizeof(C)), tile_y = r128((size_t)ny_ * TCY * sizeof(C)),
               wt = r128((size_t)nx_ * TC * sizeof(T));
  smem_ty_ = 3 * tile_y + 1024;
  smem_tconv_ = 2 * tile_x + 2 * wt + 1024;
  smem_tback_ = 3 * tile_x + 2 * wt + 1024;
  if (std::max(smem_ty_, std::max(smem_tconv_, smem_tback_)) > 220 * 1024) return false;
  raise_smem(k_cols_y_tma<T, -1, 0>, smem_ty_);
  raise_smem(k_cols_y_tma<T, +1, 0>, smem_ty_);
  raise_smem(k_xconv_tma<T, 0>, smem_tconv_);
  raise_smem(k_xbackconv_tma<T, 0>, smem_tback_);
  raise_smem(k_cols_y_tma<T, -1, 128>, smem_ty_);
  raise_smem(k_cols_y_tma<T, -1, 256>, smem_ty_);
  raise_smem(k_cols_y_tma<T, +1, 128>, smem_ty_);
  raise_smem(k_cols_y_tma<T, +1, 256>, smem_ty_);
  raise_smem(k_xconv_tma<T, 128>, smem_tconv_);
  raise_smem(k_xconv_tma<T, 256>, smem_tconv_);
  raise_smem(k_xbackconv_tma<T, 128>, smem_tback_);
  raise_smem(k_xbackconv_tma<T, 256>, smem_tback_);
  if constexpr (std::is_same<T, double>::value) {  // the double-float-spectra instances
    raise_smem(k_cols_y_tma<T, -1, 128, true>, smem_ty_);
    raise_smem(k_cols_y_tma<T, -1, 256, true>, smem_ty_);
    raise_smem(k_cols_y_tma<T, +1, 128, true>, smem_ty_);
    raise_smem(k_cols_y_tma<T, +1, 256, true>, smem_ty_);
    raise_smem(k_xconv_tma<T, 128, true>, smem_tconv_);
    raise_smem(k_xconv_tma<T, 256, true>, smem_tconv_);
    raise_smem(k_xbackconv_tma<T, 128, true>, smem_tback_);
    raise_smem(k_xbackconv_tma<T, 256, true>, smem_tback_);
  }
  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long ntile = (nzc_ + TCY - 1) / TCY;
  for (int io = 0; io < 2; ++io) {  // persistent grids from the residency of the instance launched (io: df64 spectra)
    int bps = 0;
    with_nf_io<T>(fy_, io != 0, [&](auto nf_, auto io_) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_cols_y_tma<T, -1, decltype(nf_)::value, decltype(io_)::value>, 256, smem_ty_);
    });
    bps = std::max(bps, 1);
    grid_ty1_[io] = (int)std::min<long>((long)nx_ * ntile, (long)nsm * bps);
    grid_tyM_[io] = (int)std::min<long>((long)std::max(M_, 1) * nx_ * ntile, (long)nsm * bps);
  }
  tma_ = true;
  setup_phi_tma();
  return true;
}

// The fused Phi pass: one box of RB rows of all M fields, {pz*E, RB, M}; RB
// follows the z plan (fewer rows for 256-point rows, so that three blocks fit
// an SM). Re-run whenever the z plan changes.
template <class T>
bool Evaluator<T>::setup_phi_tma() {
  tma_phi_ = false;
  constexpr int E = ElemsPerComplex<T>::value;
  const int nf = phi_nf();
  // the FP64 256-point instance copies each row group in two boxes of half a row
  const bool split = sizeof(T) == 8 && nf == 256;
  if (!tma_ || M_ == 0 || (long)pz_ * E > (split ? 512 : 256)) return false;
  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t cb = sizeof(C);
  const int RB = nf == 256 ? PhiRowsFor<T, 256>::value : PhiRowsFor<T, 128>::value;
  static_assert(PhiRowsFor<T, 128>::value == PhiRowsFor<T, 0>::value, "the runtime-plan instance groups rows as the 128-point one");
  const int L = phi_lines(M_, RB, PhiCross<T>::value);
  uint64_t dims[3] = {(uint64_t)pz_ * E, (uint64_t)rows_, (uint64_t)M_};
  uint64_t str[2] = {(uint64_t)pz_ * cb, (uint64_t)Nc_ * cb};
  uint32_t box[3] = {(uint32_t)(split ? pz_ * E / 2 : pz_ * E), (uint32_t)RB, (uint32_t)M_};
  const size_t ib = split ? 2 * r128((size_t)M_ * RB * (pz_ / 2) * cb) : r128((size_t)M_ * RB * pz_ * cb);
  smem_tphi_ = PhiBufs<T>::value * ib + 2 * r128((size_t)nz_ * (L | 1) * cb) + 1024;
  if (smem_tphi_ > 220 * 1024 || !encode_map(&mapR_, 8, Cf_, 3, dims, str, box)) return false;
  int blocks[4];  // resident blocks per SM of the Phi instances, by mode
  with_model(model_, [&](auto m) { PhiLauncher<T, decltype(m)::value>::prepare_tma(nf, ao_, smem_tphi_, blocks); });
  const long ngroup = (rows_ + RB - 1) / RB;
  grid_tphi_ = (int)std::min<long>(ngroup, (long)nsm * blocks[kPhiEval]);
  grid_thess_ = (int)std::min<long>(ngroup, (long)nsm * blocks[kPhiHess]);
  grid_tao_ = (int)std::min<long>(ngroup, (long)nsm * blocks[kPhiAO]);
  tma_phi_ = true;
  return true;
}

template <class T>
int Evaluator<T>::enable_ao(double hsdp, double reservoir, const std::vector<double>* w_ao, const double* dev_wao, cudaStream_t s,
                            std::string* err) {
  if (M_ == 0) {
    if (err) *err = "the AO model needs an FMT model";
    return 4;
  }
  if (!tma_phi_) {
    if (err) *err = "the AO model runs on the tensor-copied Phi pass, which this grid does not fit in this precision";
    return 4;
  }
  if (!w_ao && !dev_wao) return 4;
  const size_t cs = sizeof(C);
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned cgrid = (unsigned)std::min<long>(((long)M_ * Nc_ + 255) / 256, 4096);
  CK(cudaMalloc(&wao_, (size_t)M_ * Nc_ * sizeof(T)));
  if (dev_wao) {
    k_round_spectra<T><<<cgrid, 256, 0, s>>>(dev_wao, wao_, (long)M_ * Nc_);
  } else {  // the polymer weights as the colloid ones: FP64 r2c, the non-zero component, 1/N folded in
    double* tmp_real = nullptr;
    double2* tmp_spec = nullptr;
    CK(cudaMalloc(&tmp_real, N_ * sizeof(double)));
    CK(cudaMalloc(&tmp_spec, Nc_ * sizeof(double2)));
    CK(cudaMemsetAsync(tmp_spec, 0, Nc_ * sizeof(double2), s));
    const unsigned g1 = (unsigned)std::min<long>((Nc_ + 255) / 256, 4096);
    for (int a = 0; a < M_; ++a) {
      CK(cudaMemcpyAsync(tmp_real, w_ao[a].data(), N_ * sizeof(double), cudaMemcpyHostToDevice, s));
      r2c_f64(tmp_real, tmp_spec, d, tx_, ty_, tz_, s);
      k_compact<T><<<g1, 256, 0, s>>>(tmp_spec, wao_ + (long)a * Nc_, Nc_, (a >= 2 && a <= 4) ? 1 : 0, 1.0 / (double)N_);
    }
    CK(cudaStreamSynchronize(s));
    cudaFree(tmp_real);
    cudaFree(tmp_spec);
  }
  if (!NA_) CK(cudaMalloc(&NA_, (size_t)M_ * N_ * sizeof(T)));
  CK(cudaMalloc(&XA_, (size_t)M_ * N_ * sizeof(T)));
  CK(cudaMalloc(&S_, (size_t)M_ * Nc_ * cs));
  CK(cudaMemsetAsync(S_, 0, (size_t)M_ * Nc_ * cs, s));  // padding columns stay zero
  CK(cudaMalloc(&psi_, Nc_ * cs));
  CK(cudaMemsetAsync(psi_, 0, Nc_ * cs, s));
  CK(cudaMalloc(&psir_, N_ * sizeof(T)));
  gao_ = (int)std::min<long>((N_ + 255) / 256, 152 * 8);
  CK(cudaMalloc(&part_ao_, 2 * (size_t)gao_ * sizeof(double)));
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  ao_hp_ = hsdp;
  ao_res_ = reservoir;
  ao_ = true;
  // the Phi pass again, now with its AO instance (and, in FP64, on FP64 spectra: the AO
  // passes run the runtime-plan kernels, which do not take double-float spectra)
  if (!setup_phi_tma()) {
    ao_ = false;
    setup_phi_tma();  // back to the pass without the AO model
    if (err) *err = "the Phi pass with the AO model does not fit this grid";
    return 4;
  }
  return 0;
}

// The AO passes between the Phi pass (which left the polymer-folded derivative fields in
// XA and the weighted densities in NA) and the y forward pass of the derivative spectra:
// Psi = c2r(sum_a w~p_a FFT(XA_a)), e = exp(-Psi) (summed for the free energy),
// Upsilon_a = c2r(w~p_a FFT(e)), then per point reservoir x (d2Phi . Upsilon) folded for
// the colloid, whose z r2c is added to the derivative spectra in Cf: the back-convolution
// with the colloid weights then carries the AO force into dF (src/FMT.cpp:393-421).
template <class T>
void Evaluator<T>::ao_block(cudaStream_t s) {
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned gcy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_);
  const unsigned gcx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  const unsigned gr = (unsigned)grid_blocks_rows();
  const unsigned ge = (unsigned)std::min<long>((Nc_ + 255) / 256, 152 * 8);
  const unsigned gp = (unsigned)std::min<long>((N_ + 255) / 256, 152 * 8);
  auto rows_fwd = [&](const T* in, C* out) {
    with_nf(fz_, [&](auto nf_) {
      k_rows_r2c<T, T, decltype(nf_)::value><<<gr, 256, smem_rows_, s>>>(in, out, d, tz_->plan, twp<T>(tz_), rb_rows_);
    });
  };
  // spectra of the polymer-folded derivative fields
  for (int a = 0; a < M_; ++a) rows_fwd(XA_ + (long)a * N_, S_ + (long)a * Nc_);
  k_cols_fft<T, -1><<<dim3(gcy, M_), 256, smem_coly_, s>>>(S_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  k_cols_fft<T, -1><<<dim3(gcx, M_), 256, smem_colx_, s>>>(S_, Nc_, 0, d, tx_->plan, twp<T>(tx_), tc_);
  // Psi, exp(-Psi) and its sum
  k_ao_psi<T><<<ge, 256, 0, s>>>(S_, wao_, M_, Nc_, psi_);
  k_cols_fft<T, +1><<<dim3(gcx, 1), 256, smem_colx_, s>>>(psi_, Nc_, 0, d, tx_->plan, twp<T>(tx_), tc_);
  k_cols_fft<T, +1><<<dim3(gcy, 1), 256, smem_coly_, s>>>(psi_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  k_rows_c2r<T, T><<<gr, 256, smem_rows_, s>>>(psi_, psir_, d, tz_->plan, twp<T>(tz_), rb_rows_, (T)1);
  k_ao_exp<T><<<gao_, 256, 0, s>>>(psir_, N_, part_ao_);
  // Upsilon_a = w~p_a (.) FFT(exp(-Psi)), back to real space in XA
  rows_fwd(psir_, psi_);
  k_cols_fft<T, -1><<<dim3(gcy, 1), 256, smem_coly_, s>>>(psi_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  k_cols_fft<T, -1><<<dim3(gcx, 1), 256, smem_colx_, s>>>(psi_, Nc_, 0, d, tx_->plan, twp<T>(tx_), tc_);
  k_ao_upsilon<T><<<ge, 256, 0, s>>>(psi_, wao_, M_, Nc_, S_);
  k_cols_fft<T, +1><<<dim3(gcx, M_), 256, smem_colx_, s>>>(S_, Nc_, 0, d, tx_->plan, twp<T>(tx_), tc_);
  k_cols_fft<T, +1><<<dim3(gcy, M_), 256, smem_coly_, s>>>(S_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  for (int a = 0; a < M_; ++a)
    k_rows_c2r<T, T><<<gr, 256, smem_rows_, s>>>(S_ + (long)a * Nc_, XA_ + (long)a * N_, d, tz_->plan, twp<T>(tz_), rb_rows_, (T)1);
  // reservoir x (d2Phi(n) . Upsilon) per point, then its z spectra added to the derivative spectra
  const T ih = (T)(1.0 / hsd_), ih2 = (T)(1.0 / (hsd_ * hsd_)), iph = (T)(1.0 / ao_hp_), iph2 = (T)(1.0 / (ao_hp_ * ao_hp_));
  const T a = (T)esA_, b = (T)esB_, res = (T)ao_res_;
  switch (model_) {
    case MODEL_ROSENFELD: k_ao_force<T, MODEL_ROSENFELD><<<gp, 256, 0, s>>>(NA_, XA_, N_, ih, ih2, a, b, iph, iph2, res); break;
    case MODEL_RSLT: k_ao_force<T, MODEL_RSLT><<<gp, 256, 0, s>>>(NA_, XA_, N_, ih, ih2, a, b, iph, iph2, res); break;
    case MODEL_ESFMT: k_ao_force<T, MODEL_ESFMT><<<gp, 256, 0, s>>>(NA_, XA_, N_, ih, ih2, a, b, iph, iph2, res); break;
    case MODEL_WHITEBEAR_I: k_ao_force<T, MODEL_WHITEBEAR_I><<<gp, 256, 0, s>>>(NA_, XA_, N_, ih, ih2, a, b, iph, iph2, res); break;
    default: k_ao_force<T, MODEL_WHITEBEAR_II><<<gp, 256, 0, s>>>(NA_, XA_, N_, ih, ih2, a, b, iph, iph2, res); break;
  }
  for (int a2 = 0; a2 < M_; ++a2) rows_fwd(XA_ + (long)a2 * N_, S_ + (long)a2 * Nc_);
  k_spec_add<T><<<ge, 256, 0, s>>>(Cf_, S_, (long)M_ * Nc_);
}

template <class T>
int Evaluator<T>::init(int nx, int ny, int nz, int model, double hsd, double esA, double esB, const std::vector<double>* w_fmt,
                       const std::vector<double>* w_att, FFTTable* tx, FFTTable* ty, FFTTable* tz, cudaStream_t s, std::string* err,
                       const double* dev_w, const double* dev_watt) {
  nx_ = nx; ny_ = ny; nz_ = nz; nzc_ = nz / 2 + 1;
  pz_ = (nzc_ + 3) / 4 * 4;
  N_ = (long)nx * ny * nz;
  Nc_ = (long)nx * ny * pz_;
  rows_ = (long)nx * ny;
  model_ = model;
  M_ = (model < 0) ? 0 : (model >= MODEL_ESFMT ? 11 : 5);
  hsd_ = hsd; esA_ = esA; esB_ = esB;
  mf_ = (w_att != nullptr) || (dev_watt != nullptr);
  tx_ = tx; ty_ = ty; tz_ = tz;
  fixed_plans();
  Dims d{nx, ny, nz, nzc_, N_, Nc_, rows_, pz_};
  const size_t cs = sizeof(C);
  CK(cudaMalloc(&A_, Nc_ * cs));
  CK(cudaMalloc(&E_, Nc_ * cs));
  CK(cudaMemsetAsync(A_, 0, Nc_ * cs, s));
  CK(cudaMemsetAsync(E_, 0, Nc_ * cs, s));
  if (M_ > 0) {
    CK(cudaMalloc(&Cf_, (size_t)M_ * Nc_ * cs));
    CK(cudaMemsetAsync(Cf_, 0, (size_t)M_ * Nc_ * cs, s));
  }
  // launch geometry and shared memory
  smem_rows_ = smem_bytes(rb_rows_, nz, cs, 2);
  // fused phi kernel: NP lines per row; shrink rows per block to fit 200 KB
  const int NP = (M_ + 1) / 2;
  rb_phi_ = 8;
  while (rb_phi_ > 1 && (NP > 0) && smem_bytes(NP * rb_phi_, nz, cs, 2) > 200 * 1024) rb_phi_ /= 2;
  smem_phi_ = NP > 0 ? smem_bytes(NP * rb_phi_, nz, cs, 2) : 0;
  smem_colx_ = smem_bytes(tc_, nx, cs, 2);
  smem_coly_ = smem_bytes(tc_, ny, cs, 2);
  smem_xconv_ = smem_bytes(tc_, nx, cs, 3);
  smem_xback_ = smem_bytes(tc_, nx, cs, 3);
  if (std::max(std::max(smem_rows_, smem_phi_), std::max(smem_xconv_, smem_coly_)) > 220 * 1024) {
    if (err) *err = "grid too large for the shared-memory transform tiles";
    return 4;
  }
  set_smem<T>(k_rows_r2c<T, double>, smem_rows_);
  set_smem<T>(k_rows_c2r<T, double>, smem_rows_);
  set_smem<T>(k_final_rows<T, double>, smem_rows_);
  set_smem<T>(k_final_rows<T, T>, smem_rows_);
  set_smem<T>(k_rows_r2c<T, T>, smem_rows_);
  set_smem<T>(k_final_rows<T, double, 128>, smem_rows_);
  set_smem<T>(k_final_rows<T, double, 256>, smem_rows_);
  set_smem<T>(k_final_rows<T, T, 128>, smem_rows_);
  set_smem<T>(k_final_rows<T, T, 256>, smem_rows_);
  set_smem<T>(k_rows_r2c<T, T, 128>, smem_rows_);
  set_smem<T>(k_rows_r2c<T, double, 128>, smem_rows_);
  set_smem<T>(k_rows_r2c<T, T, 256>, smem_rows_);
  set_smem<T>(k_rows_r2c<T, double, 256>, smem_rows_);
  set_smem<T>(k_cols_fft<T, -1>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_cols_fft<T, +1>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_cols_fft<T, -1, 128>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_cols_fft<T, +1, 128>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_cols_fft<T, -1, 256>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_cols_fft<T, +1, 256>, std::max(smem_colx_, smem_coly_));
  set_smem<T>(k_rows_c2r<T, double, 128>, smem_rows_);
  set_smem<T>(k_rows_c2r<T, double, 256>, smem_rows_);
  set_smem<T>(k_xconv<T>, smem_xconv_);
  set_smem<T>(k_xbackconv<T>, smem_xback_);
  if (M_ > 0) with_model(model_, [&](auto m) { PhiLauncher<T, decltype(m)::value>::prepare_rows(smem_phi_); });
  set_smem<T>(k_rows_c2r<T, T>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, double>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, T>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, double, 128>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, T, 128>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, double, 256>, smem_rows_);
  set_smem<T>(k_hess_final_rows<T, T, 256>, smem_rows_);
  if constexpr (std::is_same<T, double>::value) {  // the double-float-spectra instances
    set_smem<T>(k_rows_r2c<T, double, 128, true>, smem_rows_);
    set_smem<T>(k_rows_r2c<T, double, 256, true>, smem_rows_);
    set_smem<T>(k_final_rows<T, double, 128, true>, smem_rows_);
    set_smem<T>(k_final_rows<T, double, 256, true>, smem_rows_);
    set_smem<T>(k_hess_final_rows<T, double, 128, true>, smem_rows_);
    set_smem<T>(k_hess_final_rows<T, double, 256, true>, smem_rows_);
  }
  // partial-sum storage: phi blocks (1 value), x columns (1 value), final rows (4 values)
  const long ncolx = ((long)ny * pz_ + 7) / 8 + 16;  // x-pass blocks of the widest grid (8 columns per tile)
  // phi partials: at most one per row (both the row-group and the persistent grids stay below it)
  part_len_ = 2 * (rows_ + ncolx + 4 * grid_blocks_rows());
  CK(cudaMalloc(&part_, part_len_ * sizeof(double)));
  CK(cudaMalloc(&terms_, 8 * sizeof(double)));
  CK(cudaMalloc(&status_, sizeof(unsigned)));
  CK(cudaMemsetAsync(terms_, 0, 8 * sizeof(double), s));
  if (M_ > 0 && dev_w) {  // weight spectra rounded from an FP64 evaluator's
    const unsigned cg = (unsigned)std::min<long>(((long)M_ * Nc_ + 255) / 256, 4096);
    CK(cudaMalloc(&w_, (size_t)M_ * Nc_ * sizeof(T)));
    k_round_spectra<T><<<cg, 256, 0, s>>>(dev_w, w_, (long)M_ * Nc_);
  }
  if (mf_ && dev_watt) {
    const unsigned cg = (unsigned)std::min<long>((Nc_ + 255) / 256, 4096);
    CK(cudaMalloc(&watt_, Nc_ * sizeof(T)));
    k_round_spectra<T><<<cg, 256, 0, s>>>(dev_watt, watt_, Nc_);
  }
  if ((M_ == 0 || dev_w) && (!mf_ || dev_watt)) {
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    if (!setup_tma(err)) tma_ = false;
    return 0;
  }
  // weight spectra: FP64 r2c on the device, keep the non-zero component, fold 1/N
  double* tmp_real = nullptr;
  double2* tmp_spec = nullptr;
  CK(cudaMalloc(&tmp_real, N_ * sizeof(double)));
  CK(cudaMalloc(&tmp_spec, Nc_ * sizeof(double2)));
  CK(cudaMemsetAsync(tmp_spec, 0, Nc_ * sizeof(double2), s));
  const unsigned cgrid = (unsigned)std::min<long>((Nc_ + 255) / 256, 4096);
  if (M_ > 0 && !dev_w) {
    CK(cudaMalloc(&w_, (size_t)M_ * Nc_ * sizeof(T)));
    CK(cudaMemsetAsync(w_, 0, (size_t)M_ * Nc_ * sizeof(T), s));
    for (int a = 0; a < M_; ++a) {
      CK(cudaMemcpyAsync(tmp_real, w_fmt[a].data(), N_ * sizeof(double), cudaMemcpyHostToDevice, s));
      r2c_f64(tmp_real, tmp_spec, d, tx, ty, tz, s);
      k_compact<T><<<cgrid, 256, 0, s>>>(tmp_spec, w_ + (long)a * Nc_, Nc_, (a >= 2 && a <= 4) ? 1 : 0, 1.0 / (double)N_);
    }
  }
  if (mf_ && !dev_watt) {
    CK(cudaMalloc(&watt_, Nc_ * sizeof(T)));
    CK(cudaMemcpyAsync(tmp_real, w_att->data(), N_ * sizeof(double), cudaMemcpyHostToDevice, s));
    r2c_f64(tmp_real, tmp_spec, d, tx, ty, tz, s);
    k_compact<T><<<cgrid, 256, 0, s>>>(tmp_spec, watt_, Nc_, 0, 1.0 / (double)N_);
  }
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  cudaFree(tmp_real);
  cudaFree(tmp_spec);
  if (!setup_tma(err)) tma_ = false;
  return 0;
}

template <class T>
void Evaluator<T>::r2c(const double* in, C* out, cudaStream_t s) {
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned gy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_), gx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  with_nf(fz_, [&](auto nf_) {
    k_rows_r2c<T, double, decltype(nf_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(in, out, d, tz_->plan, twp<T>(tz_),
                                                                                                    rb_rows_);
  });
  with_nf(fy_, [&](auto nf_) {
    k_cols_fft<T, -1, decltype(nf_)::value><<<dim3(gy, 1), 256, smem_coly_, s>>>(out, 0, 1, d, ty_->plan, twp<T>(ty_), tc_);
  });
  with_nf(fx_, [&](auto nf_) {
    k_cols_fft<T, -1, decltype(nf_)::value><<<dim3(gx, 1), 256, smem_colx_, s>>>(out, 0, 0, d, tx_->plan, twp<T>(tx_), tc_);
  });
}

template <class T>
void Evaluator<T>::c2r(const C* in, double* out, T scale, cudaStream_t s) {
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned gy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_), gx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  C* work = E_;  // scratch between evaluations (the next evaluation rewrites it)
  cudaMemcpyAsync(work, in, Nc_ * sizeof(C), cudaMemcpyDeviceToDevice, s);
  with_nf(fx_, [&](auto nf_) {
    k_cols_fft<T, +1, decltype(nf_)::value><<<dim3(gx, 1), 256, smem_colx_, s>>>(work, 0, 0, d, tx_->plan, twp<T>(tx_), tc_);
  });
  with_nf(fy_, [&](auto nf_) {
    k_cols_fft<T, +1, decltype(nf_)::value><<<dim3(gy, 1), 256, smem_coly_, s>>>(work, 0, 1, d, ty_->plan, twp<T>(ty_), tc_);
  });
  with_nf(fz_, [&](auto nf_) {
    k_rows_c2r<T, double, decltype(nf_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(work, out, d, tz_->plan, twp<T>(tz_),
                                                                                                    rb_rows_, scale);
  });
}

template <class T>
template <class RT>
int Evaluator<T>::launch(const RT* rho, const double* vext, RT* dF, double dV, double mu, int ideal, cudaStream_t s, cudaEvent_t* ev,
                         double* nrm, RT* dF_mirror) {
  auto mark = [&](int i) {
    if (ev) cudaEventRecord(ev[i], s);
  };
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  constexpr int TCt = TileCols<T>::value;
  const unsigned gcy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_);
  const unsigned gcx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  const unsigned gtx = (unsigned)(((long)ny_ * pz_ + TCt - 1) / TCt);
  const unsigned gxb = tma_ ? gtx : gcx;
  const long nphi = (rows_ + rb_phi_ - 1) / rb_phi_;
  double* part_phi = part_;
  double* part_mf = part_ + 2 * rows_;
  double* part_fin = part_mf + 2 * (long)std::max(gcx, gtx);
  const bool any = M_ > 0 || mf_;
  const bool io = df_spectra();
  auto yfwd = [&](C* buf, const CUtensorMap& map, int nf, int grid) {
    if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, -1, decltype(nf_)::value, decltype(io_)::value><<<grid, 256, smem_ty_, s>>>(map, d, ty_->plan, twp<T>(ty_), nf, status_); });
    else k_cols_fft<T, -1><<<dim3(gcy, nf), 256, smem_coly_, s>>>(buf, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  };
  auto yinv = [&](C* buf, const CUtensorMap& map, int nf, int grid) {
    if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, +1, decltype(nf_)::value, decltype(io_)::value><<<grid, 256, smem_ty_, s>>>(map, d, ty_->plan, twp<T>(ty_), nf, status_); });
    else k_cols_fft<T, +1><<<dim3(gcy, nf), 256, smem_coly_, s>>>(buf, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  };
  cudaMemsetAsync(status_, 0, sizeof(unsigned), s);
  mark(0);
  if (any) {
    with_nf_io<T>(fz_, io, [&](auto nf_, auto io_) {
      k_rows_r2c<T, RT, decltype(nf_)::value, decltype(io_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(rho, A_, d, tz_->plan,
                                                                                                                        twp<T>(tz_), rb_rows_);
    });
    mark(1);
    yfwd(A_, mapYA_, 1, grid_ty1_[io]);
    mark(2);
  } else {
    mark(1);
    mark(2);
  }
  if (M_ > 0) {
    if (tma_) with_nf_io<T>(fx_, io, [&](auto nf_, auto io_) { k_xconv_tma<T, decltype(nf_)::value, decltype(io_)::value><<<gtx, 256, smem_tconv_, s>>>(mapA_, decltype(io_)::value ? mapWdf_ : mapW_, mapCf_, M_, tx_->plan, twp<T>(tx_), status_); });
    else k_xconv<T><<<gcx, 256, smem_xconv_, s>>>(A_, Cf_, w_, M_, d, tx_->plan, twp<T>(tx_), tc_);
    mark(3);
    yinv(Cf_, mapYC_, M_, grid_tyM_[io]);
    mark(4);
    PhiArgs pa;
    pa.map = &mapR_;
    pa.Cf = Cf_;
    pa.d = d;
    pa.plan = tz_->plan;
    pa.tw = twp<T>(tz_);
    pa.hsd = hsd_;
    pa.esA = esA_;
    pa.esB = esB_;
    pa.part = part_phi;
    pa.status = status_;
    pa.NA = NA_;
    pa.XA = XA_;
    if (ao_) {
      pa.iph = 1.0 / ao_hp_;
      pa.iph2 = 1.0 / (ao_hp_ * ao_hp_);
    }
    if (tma_phi_) {  // FMT_AO_Species: the Phi pass also leaves NA and the polymer-folded fields
      phi_blocks_last_ = ao_ ? grid_tao_ : grid_tphi_;
      with_model(model_, [&](auto m) {
        PhiLauncher<T, decltype(m)::value>::launch_tma(phi_nf(), ao_ ? kPhiAO : kPhiEval, pa, (int)phi_blocks_last_, smem_tphi_, s);
      });
      if (ao_) ao_block(s);
    } else {
      phi_blocks_last_ = nphi;
      with_model(model_, [&](auto m) { PhiLauncher<T, decltype(m)::value>::launch_rows(false, pa, rb_phi_, (unsigned)nphi, smem_phi_, s); });
    }
    mark(5);
    yfwd(Cf_, mapYC_, M_, grid_tyM_[io]);
    mark(6);
  } else {
    for (int i = 3; i <= 6; ++i) mark(i);
  }
  if (any) {
    if (tma_)
      with_nf_io<T>(fx_, io, [&](auto nf_, auto io_) {
        k_xbackconv_tma<T, decltype(nf_)::value, decltype(io_)::value><<<gtx, 256, smem_tback_, s>>>(
            mapCf_, decltype(io_)::value ? mapWdf_ : mapW_, mapA_, decltype(io_)::value ? mapWattdf_ : mapWatt_, mapE_, M_, mf_ ? 1 : 0, d,
            tx_->plan, twp<T>(tx_), mf_ ? part_mf : nullptr, status_);
      });
    else
      k_xbackconv<T><<<gcx, 256, smem_xback_, s>>>(Cf_, A_, E_, w_, mf_ ? watt_ : nullptr, M_, d, tx_->plan, twp<T>(tx_), tc_,
                                                   mf_ ? part_mf : nullptr);
    mark(7);
    yinv(E_, mapYE_, 1, grid_ty1_[io]);
    mark(8);
  } else {
    mark(7);
    mark(8);
  }
  const unsigned gfin = (unsigned)grid_blocks_rows();
  with_nf_io<T>(fz_, io, [&](auto nf_, auto io_) {
    k_final_rows<T, RT, decltype(nf_)::value, decltype(io_)::value><<<gfin, 256, smem_rows_, s>>>(E_, rho, vext, dF, d, tz_->plan, twp<T>(tz_),
                                                                                                 rb_rows_, dV, mu, any ? 1 : 0, ideal, part_fin, nrm,
                                                                                                 dF_mirror);
  });
  {
    const FinishSeg sphi{part_phi, phi_blocks_last_, M_ > 0 ? 1 : 0, terms_ + 0};
    const FinishSeg smf{part_mf, (long)gxb, mf_ ? 1 : 0, terms_ + 1};
    const FinishSeg sfin{part_fin, (long)gfin, 4, terms_ + 2};
    const FinishSeg sao{part_ao_, (long)gao_, ao_ ? 1 : 0, terms_ + 6};
    k_finish_terms<<<1, 224, 0, s>>>(sphi, smf, sfin, sao);
  }
  mark(9);
  return 0;
}

// ------------------------------------------------------------ Hessian ---
template <class T>
int Evaluator<T>::hess_prepare(const double* rho0, cudaStream_t s) {
  if (M_ == 0) return 0;
  if (!NA_ && cudaMalloc(&NA_, (size_t)M_ * N_ * sizeof(T)) != cudaSuccess) return 5;
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned gcy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_);
  const unsigned gcx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  constexpr int TCt = TileCols<T>::value;
  const unsigned gtx = (unsigned)(((long)ny_ * pz_ + TCt - 1) / TCt);
  const bool io = df_spectra();
  with_nf_io<T>(fz_, io, [&](auto nf_, auto io_) {
    k_rows_r2c<T, double, decltype(nf_)::value, decltype(io_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(
        rho0, A_, d, tz_->plan, twp<T>(tz_), rb_rows_);
  });
  if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, -1, decltype(nf_)::value, decltype(io_)::value><<<grid_ty1_[io], 256, smem_ty_, s>>>(mapYA_, d, ty_->plan, twp<T>(ty_), 1, status_); });
  else k_cols_fft<T, -1><<<dim3(gcy, 1), 256, smem_coly_, s>>>(A_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  if (tma_) with_nf_io<T>(fx_, io, [&](auto nf_, auto io_) { k_xconv_tma<T, decltype(nf_)::value, decltype(io_)::value><<<gtx, 256, smem_tconv_, s>>>(mapA_, decltype(io_)::value ? mapWdf_ : mapW_, mapCf_, M_, tx_->plan, twp<T>(tx_), status_); });
  else k_xconv<T><<<gcx, 256, smem_xconv_, s>>>(A_, Cf_, w_, M_, d, tx_->plan, twp<T>(tx_), tc_);
  if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, +1, decltype(nf_)::value, decltype(io_)::value><<<grid_tyM_[io], 256, smem_ty_, s>>>(mapYC_, d, ty_->plan, twp<T>(ty_), M_, status_); });
  else k_cols_fft<T, +1><<<dim3(gcy, M_), 256, smem_coly_, s>>>(Cf_, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  PhiArgs pa;
  pa.map = &mapR_;
  pa.Cf = Cf_;
  pa.d = d;
  pa.plan = tz_->plan;
  pa.tw = twp<T>(tz_);
  pa.hsd = hsd_;
  pa.esA = esA_;
  pa.esB = esB_;
  pa.status = status_;
  pa.NA = NA_;
  if (tma_phi_) {  // one tensor-copied pass: z c2r of all M fields, stored as the weighted densities
    with_model(model_, [&](auto m) { PhiLauncher<T, decltype(m)::value>::launch_tma(phi_nf(), kPhiStoreN, pa, grid_tphi_, smem_tphi_, s); });
  } else {
    for (int a = 0; a < M_; ++a)
      k_rows_c2r<T, T><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(Cf_ + (long)a * Nc_, NA_ + (long)a * N_, d, tz_->plan,
                                                                             twp<T>(tz_), rb_rows_, (T)1);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : 5;
}

template <class T>
template <class RT>
int Evaluator<T>::hess_apply(const RT* v, const double* rho0, RT* out, double dV, cudaStream_t s) {
  if (M_ > 0 && !NA_) return 7;
  Dims d{nx_, ny_, nz_, nzc_, N_, Nc_, rows_, pz_};
  const unsigned gcy = (unsigned)(((long)nx_ * nzc_ + tc_ - 1) / tc_);
  const unsigned gcx = (unsigned)(((long)ny_ * pz_ + tc_ - 1) / tc_);
  constexpr int TCt = TileCols<T>::value;
  const unsigned gtx = (unsigned)(((long)ny_ * pz_ + TCt - 1) / TCt);
  const bool any = M_ > 0 || mf_;
  const bool io = df_spectra();
  auto yfwd = [&](C* buf, const CUtensorMap& map, int nf, int grid) {
    if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, -1, decltype(nf_)::value, decltype(io_)::value><<<grid, 256, smem_ty_, s>>>(map, d, ty_->plan, twp<T>(ty_), nf, status_); });
    else k_cols_fft<T, -1><<<dim3(gcy, nf), 256, smem_coly_, s>>>(buf, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  };
  auto yinv = [&](C* buf, const CUtensorMap& map, int nf, int grid) {
    if (tma_) with_nf_io<T>(fy_, io, [&](auto nf_, auto io_) { k_cols_y_tma<T, +1, decltype(nf_)::value, decltype(io_)::value><<<grid, 256, smem_ty_, s>>>(map, d, ty_->plan, twp<T>(ty_), nf, status_); });
    else k_cols_fft<T, +1><<<dim3(gcy, nf), 256, smem_coly_, s>>>(buf, Nc_, 1, d, ty_->plan, twp<T>(ty_), tc_);
  };
  if (any) {
    with_nf_io<T>(fz_, io, [&](auto nf_, auto io_) {
      k_rows_r2c<T, RT, decltype(nf_)::value, decltype(io_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(v, A_, d, tz_->plan, twp<T>(tz_), rb_rows_);
    });
    yfwd(A_, mapYA_, 1, grid_ty1_[io]);
  }
  if (M_ > 0) {
    if (tma_) with_nf_io<T>(fx_, io, [&](auto nf_, auto io_) { k_xconv_tma<T, decltype(nf_)::value, decltype(io_)::value><<<gtx, 256, smem_tconv_, s>>>(mapA_, decltype(io_)::value ? mapWdf_ : mapW_, mapCf_, M_, tx_->plan, twp<T>(tx_), status_); });
    else k_xconv<T><<<gcx, 256, smem_xconv_, s>>>(A_, Cf_, w_, M_, d, tx_->plan, twp<T>(tx_), tc_);
    yinv(Cf_, mapYC_, M_, grid_tyM_[io]);
    const unsigned g = (unsigned)((rows_ + rb_phi_ - 1) / rb_phi_);
    PhiArgs pa;
    pa.map = &mapR_;
    pa.Cf = Cf_;
    pa.d = d;
    pa.plan = tz_->plan;
    pa.tw = twp<T>(tz_);
    pa.hsd = hsd_;
    pa.esA = esA_;
    pa.esB = esB_;
    pa.status = status_;
    pa.NA = NA_;
    with_model(model_, [&](auto m) {
      if (tma_phi_) PhiLauncher<T, decltype(m)::value>::launch_tma(phi_nf(), kPhiHess, pa, grid_thess_, smem_tphi_, s);
      else PhiLauncher<T, decltype(m)::value>::launch_rows(true, pa, rb_phi_, g, smem_phi_, s);
    });
    yfwd(Cf_, mapYC_, M_, grid_tyM_[io]);
  }
  double* part_mf = part_ + 2 * rows_;
  if (any) {
    if (tma_)
      with_nf_io<T>(fx_, io, [&](auto nf_, auto io_) {
        k_xbackconv_tma<T, decltype(nf_)::value, decltype(io_)::value><<<gtx, 256, smem_tback_, s>>>(
            mapCf_, decltype(io_)::value ? mapWdf_ : mapW_, mapA_, decltype(io_)::value ? mapWattdf_ : mapWatt_, mapE_, M_, mf_ ? 1 : 0, d,
            tx_->plan, twp<T>(tx_), mf_ ? part_mf : nullptr, status_);
      });
    else
      k_xbackconv<T><<<gcx, 256, smem_xback_, s>>>(Cf_, A_, E_, w_, mf_ ? watt_ : nullptr, M_, d, tx_->plan, twp<T>(tx_), tc_,
                                                   mf_ ? part_mf : nullptr);
    yinv(E_, mapYE_, 1, grid_ty1_[io]);
  }
  with_nf_io<T>(fz_, io, [&](auto nf_, auto io_) {
    k_hess_final_rows<T, RT, decltype(nf_)::value, decltype(io_)::value><<<(unsigned)grid_blocks_rows(), 256, smem_rows_, s>>>(
        E_, rho0, v, out, d, tz_->plan, twp<T>(tz_), rb_rows_, dV, any ? 1 : 0);
  });
  return cudaGetLastError() == cudaSuccess ? 0 : 5;
}

template <class T>
void Evaluator<T>::fixed_plans() {
  // the compile-time plan length of an axis: 128 or 256 with the default radix order, else 0
  auto fixed_len = [](const FFTTable* t) {
    if (!t || (t->plan.n != 128 && t->plan.n != 256)) return 0;
    const std::vector<int> d = default_radices(t->plan.n);
    if ((int)d.size() != t->plan.nst) return 0;
    for (int i = 0; i < t->plan.nst; ++i)
      if (t->plan.radix[i] != d[i]) return 0;
    return t->plan.n;
  };
  fx_ = fixed_len(tx_);
  fy_ = fixed_len(ty_);
  fz_ = fixed_len(tz_);
}

template <class T>
bool Evaluator<T>::df_candidate() const {
  return kDf64Transforms && std::is_same<T, double>::value && fx_ > 0 && fy_ > 0 && fz_ > 0 && tma_ && !ao_ && M_ > 0 && wdf_ &&
         (!mf_ || wattdf_);
}

template <class T>
int Evaluator<T>::phi_nf() const {
  return (kDf64Transforms && std::is_same<T, double>::value && !df_candidate()) ? 0 : fz_;
}

template <class T>
void Evaluator<T>::pass_bytes(double* by) const {
  const double b = sizeof(T), N = (double)N_, Nc = (double)nx_ * ny_ * nzc_, M = M_;
  const double C = 2 * Nc * b, W = Nc * b;
  const bool any = M_ > 0 || mf_;
  by[0] = any ? N * 8 + C : 0;                        // rows_r2c: rho (f64) -> A
  by[1] = any ? 2 * C : 0;                            // y forward of A
  by[2] = M_ ? C + M * W + M * C : 0;                 // xconv: A, weights -> C[a]
  by[3] = M_ ? M * 2 * C : 0;                         // y inverse of C[a]
  by[4] = M_ ? M * 2 * C : 0;                         // phi rows: C[a] -> D[a]
  by[5] = M_ ? M * 2 * C : 0;                         // y forward of D[a]
  by[6] = any ? M * (C + W) + (mf_ ? C + W : 0) + C : 0;  // xbackconv: D[a], weights, A, w_att -> E
  by[7] = any ? 2 * C : 0;                            // y inverse of E
  by[8] = (any ? C : 0) + 2 * N * 8;                  // final rows: E, rho (f64) -> dF (f64)
}

template <class T>
int Evaluator<T>::finish(double dV, double mu, EvalTerms* out, cudaStream_t s) {
  double h[8];
  unsigned st = 0;
  cudaMemcpyAsync(h, terms_, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&st, status_, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return 5;
  return terms_from(h, st, dV, mu, out);
}

template <class T>
int Evaluator<T>::terms_from(const double* h, unsigned st, double dV, double mu, EvalTerms* out) const {
  out->F_hs = M_ > 0 ? h[0] * dV : 0.0;
  // FMT_AO_Species::free_energy_post_process (src/FMT_Species.cpp:694-738): rho_p (N - sum exp(-Psi)), x dV
  if (ao_) out->F_hs = (h[0] + ao_res_ * ((double)N_ - h[6])) * dV;
  out->F_mf = mf_ ? 0.5 * dV * h[1] : 0.0;
  out->F_id = h[2];
  out->sum_rho = h[3];
  out->sum_vext_rho = h[4];
  out->sum_dF_rho = h[5];
  out->F_ext = h[4] * dV - (h[3] * dV) * mu;
  out->status = st;
  if (st & kStatusTimeout) return 3;
  out->Omega = ((out->F_id + out->F_hs) + out->F_mf) + out->F_ext;
  return (cudaGetLastError() == cudaSuccess) ? 0 : 5;
}

template <class T>
int Evaluator<T>::eval(const double* rho, const double* vext, double* dF, double dV, double mu, int ideal, EvalTerms* out, cudaStream_t s) {
  int rc = launch(rho, vext, dF, dV, mu, ideal, s);
  if (rc) return rc;
  return finish(dV, mu, out, s);
}

template class Evaluator<float>;
template class Evaluator<double>;
template int Evaluator<float>::launch<float>(const float*, const double*, float*, double, double, int, cudaStream_t, cudaEvent_t*,
                                             double*, float*);
template int Evaluator<float>::hess_apply<float>(const float*, const double*, float*, double, cudaStream_t);
template int Evaluator<float>::hess_apply<double>(const double*, const double*, double*, double, cudaStream_t);
template int Evaluator<double>::hess_apply<double>(const double*, const double*, double*, double, cudaStream_t);

}  // namespace cdft

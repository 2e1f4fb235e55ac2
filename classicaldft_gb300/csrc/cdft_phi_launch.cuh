// Definitions of PhiLauncher (cdft_phi_launch.h), included only by the per-model units.
#pragma once
#include <algorithm>
#include "cdft_phi_launch.h"

namespace cdft {

namespace phi_detail {
template <class F>
inline void raise(F f, size_t bytes) {  // never lowers a limit another context launches with
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, f) == cudaSuccess && (size_t)a.maxDynamicSharedSizeBytes >= bytes) return;
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
template <class F>
inline int resident(F f, int threads, size_t bytes) {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, threads, bytes);
  return std::max(b, 1);
}
template <class T, class F>
inline void with_phi_nf(int nf, F&& f) {
  if (nf == 128) f(std::integral_constant<int, 128>());
  else if (nf == 256) f(std::integral_constant<int, 256>());
  else f(std::integral_constant<int, 0>());
}
}  // namespace phi_detail

template <class T, int MODEL>
void PhiLauncher<T, MODEL>::prepare_tma(int nf, bool ao, size_t smem, int blocks[4]) {
  phi_detail::with_phi_nf<T>(nf, [&](auto nf_) {
    constexpr int NF = decltype(nf_)::value, RB = PhiRowsFor<T, NF>::value, NT = PhiThreads<T>::value;
    auto one = [&](auto kern) {
      phi_detail::raise(kern, smem);
      return phi_detail::resident(kern, NT, smem);
    };
    blocks[kPhiEval] = one(k_phi_rows_tma<T, MODEL, RB, NF, kPhiEval>);
    blocks[kPhiHess] = one(k_phi_rows_tma<T, MODEL, RB, NF, kPhiHess>);
    blocks[kPhiStoreN] = one(k_phi_rows_tma<T, MODEL, RB, NF, kPhiStoreN>);
    blocks[kPhiAO] = ao ? one(k_phi_rows_tma<T, MODEL, RB, NF, kPhiAO>) : 1;
  });
}

template <class T, int MODEL>
void PhiLauncher<T, MODEL>::launch_tma(int nf, int mode, const PhiArgs& a, int grid, size_t smem, cudaStream_t s) {
  typedef typename Cx<T>::type C;
  C* Cf = static_cast<C*>(a.Cf);
  const C* tw = static_cast<const C*>(a.tw);
  T* NA = static_cast<T*>(a.NA);
  T* XA = static_cast<T*>(a.XA);
  const T h = (T)a.hsd, A = (T)a.esA, B = (T)a.esB;
  phi_detail::with_phi_nf<T>(nf, [&](auto nf_) {
    constexpr int NF = decltype(nf_)::value, RB = PhiRowsFor<T, NF>::value, NT = PhiThreads<T>::value;
    switch (mode) {
      case kPhiEval:
        k_phi_rows_tma<T, MODEL, RB, NF, kPhiEval><<<grid, NT, smem, s>>>(*a.map, Cf, a.d, a.plan, tw, h, A, B, a.part, a.status);
        break;
      case kPhiHess:
        k_phi_rows_tma<T, MODEL, RB, NF, kPhiHess><<<grid, NT, smem, s>>>(*a.map, Cf, a.d, a.plan, tw, h, A, B, nullptr, a.status, NA);
        break;
      case kPhiStoreN:
        k_phi_rows_tma<T, MODEL, RB, NF, kPhiStoreN><<<grid, NT, smem, s>>>(*a.map, Cf, a.d, a.plan, tw, h, A, B, nullptr, a.status, NA);
        break;
      default:
        k_phi_rows_tma<T, MODEL, RB, NF, kPhiAO><<<grid, NT, smem, s>>>(*a.map, Cf, a.d, a.plan, tw, h, A, B, a.part, a.status, NA, XA,
                                                                        (T)a.iph, (T)a.iph2);
        break;
    }
  });
}

template <class T, int MODEL>
void PhiLauncher<T, MODEL>::prepare_rows(size_t smem) {
  phi_detail::raise(k_phi_rows<T, MODEL>, smem);
  phi_detail::raise(k_hess_rows<T, MODEL>, smem);
}

template <class T, int MODEL>
void PhiLauncher<T, MODEL>::launch_rows(bool hess, const PhiArgs& a, int rb, unsigned grid, size_t smem, cudaStream_t s) {
  typedef typename Cx<T>::type C;
  C* Cf = static_cast<C*>(a.Cf);
  const C* tw = static_cast<const C*>(a.tw);
  const T h = (T)a.hsd, A = (T)a.esA, B = (T)a.esB;
  if (hess)
    k_hess_rows<T, MODEL><<<grid, 256, smem, s>>>(Cf, static_cast<const T*>(a.NA), a.d, a.plan, tw, rb, h, A, B);
  else
    k_phi_rows<T, MODEL><<<grid, 256, smem, s>>>(Cf, a.d, a.plan, tw, rb, h, A, B, a.part, a.status);
}

}  // namespace cdft

#define CDFT_PHI_INSTANTIATE(MODEL)                    \
  namespace cdft {                                     \
  template struct PhiLauncher<float, MODEL>;           \
  template struct PhiLauncher<double, MODEL>;          \
  }

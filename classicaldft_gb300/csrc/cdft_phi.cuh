// Pointwise FMT free-energy density Phi and its derivatives for one species,
// folded into the per-species weighted-density derivatives used by the
// back-convolution. Follows FMT::calculate_Phi / calculate_dPhi_wrt_fundamental_measures
// (src/FMT.cpp:114-176), the model functions f1/f2/f3 and Phi3 of
// include/FMT.h:139-643, and FMT_Species::set_fundamental_measure_derivatives
// (include/Species.h:310-329): dPhi_s = dPhi_s0/d^2 + dPhi_s1/d + dPhi_s2, the
// vector derivative carries the parity sign, off-diagonal tensor terms x2.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "cdft_df64.cuh"
#include "cdft_types.h"

namespace cdft {

template <int MODEL> struct ModelTraits { static constexpr bool tensor = MODEL >= MODEL_ESFMT; static constexpr int M = tensor ? 11 : 5; };

template <class T> __device__ __forceinline__ T log1m(T e);
template <> __device__ __forceinline__ double log1m<double>(double e) { return log(1.0 - e); }
template <> __device__ __forceinline__ float log1m<float>(float e) { return log1pf(-e); }
// df64: table-driven log1p on the FP32 pipe (the kernel initialises df_log_table first)
template <> __device__ __forceinline__ dfs log1m<dfs>(dfs e) { return df_log1p(-e); }
template <> __device__ __forceinline__ dfl log1m<dfl>(dfl e) { return dfl(df_log1p(-e.norm())); }
// natural logarithm in the argument's own precision (logf for FP32, never a promotion to FP64)
template <class T> __device__ __forceinline__ T ln_t(T x);
template <> __device__ __forceinline__ double ln_t<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float ln_t<float>(float x) { return logf(x); }
// exponential in the argument's own precision
template <class T> __device__ __forceinline__ T exp_t(T x);
template <> __device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }

// f1, f2, f3 and first derivatives. Divisions are replaced by products with
// g = 1/(1 - eta) and ie = 1/eta: GB300 runs FP64 division as a long FP64
// instruction sequence, so WhiteBear I and RSLT take both from one division.
template <class T, int MODEL>
__device__ __forceinline__ void fmt_f(T e, T& f1, T& f2, T& f3, T& f1p, T& f2p, T& f3p) {
  const T one = (T)1;
  const T L = log1m<T>(e);
  if (MODEL == MODEL_RSLT || MODEL == MODEL_WHITEBEAR_I) {
    // one division for both reciprocals away from eta = 0: q = 1/(eta (1 - eta)),
    // 1/(1 - eta) = eta q, 1/eta = (1 - eta) q
    const T om = one - e;
    T g, ie = 0;
    const bool small = e < (T)1e-12;
    if (small) {
      g = one / om;
    } else {
      const T q = one / (e * om);
      g = e * q;
      ie = om * q;
    }
    f1 = L;
    f1p = -g;
    f2 = g;
    f2p = g * g;
    if (small) {
      f3 = (T)1.5 + (T)(8.0 / 3) * e + (T)3.75 * e * e + (T)4.8 * e * e * e;
      f3p = (T)(8.0 / 3) + (T)7.5 * e + (T)14.4 * e * e;
    } else {
      const T g2 = g * g;
      f3 = ie * g2 + L * ie * ie;
      if (MODEL == MODEL_RSLT)
        f3p = -ie * ie * g2 * g * (e * e - (T)5 * e + (T)2) - (T)2 * ie * ie * ie * L;
      else
        f3p = (-(T)2 + (T)5 * e - e * e) * ie * ie * g2 * g - (T)2 * ie * ie * ie * L;
    }
    return;
  }
  const T g = one / (one - e);
  f1 = L;
  f1p = -g;
  if (MODEL == MODEL_WHITEBEAR_II) {
    if (e < (T)1e-12) {
      f2 = one + e * (one + e * ((T)(10.0 / 9) + (T)(7.0 / 6) * e));
      f2p = one + e * ((T)(20.0 / 9) + (T)3.5 * e);
      f3 = (T)1.5 + (T)(7.0 / 3) * e + (T)3.25 * e * e + (T)4.2 * e * e * e;
      f3p = (T)(7.0 / 3) + (T)7.5 * e + (T)12.6 * e * e;
    } else {
      const T ie = one / e, g2 = g * g;
      f2 = (T)(1.0 / 3.0) + (T)(4.0 / 3.0) * g + (T)(2.0 / 3.0) * ie * L;
      f2p = (T)(2.0 / 3.0) * ((T)3 * e - one) * ie * g2 - (T)(2.0 / 3.0) * ie * ie * L;
      f3 = -(one - (T)3 * e + e * e) * ie * g2 - ie * ie * L;
      f3p = ((T)2 - (T)5 * e + (T)6 * e * e - e * e * e) * ie * ie * g2 * g + (T)2 * ie * ie * ie * L;
    }
    return;
  }
  // Rosenfeld and esFMT
  f2 = g;
  f2p = g * g;
  f3 = g * g;
  f3p = (T)2 * g * g * g;
}

// The same f-functions for a df64 eta (the FP64 Phi pass keeps its values in df64): the
// same formulas in df64, the logarithm and the reciprocals too (cdft_df64.cuh), so the
// pass runs no FP64 arithmetic per point. The kernel initialises df_log_table first.
template <int MODEL>
__device__ __forceinline__ void fmt_f_df(dfs e, dfs& f1, dfs& f2, dfs& f3, dfs& f1p, dfs& f2p, dfs& f3p) {
  fmt_f<dfs, MODEL>(e, f1, f2, f3, f1p, f2p, f3p);
}

// n[] holds the weighted densities in the order eta, s, v0, v1, v2, T00, T01,
// T02, T11, T12, T22 (M = 11) or the first five (M = 5). On return n[] holds
// dPhi/dn_a folded as described above. Returns Phi. ih = 1/hsd, ih2 = 1/hsd^2.
// ao (optional): the s and v slots folded with the polymer diameter d_p instead
// (ao[0] = dPhi/ds0 / d_p^2 + dPhi/ds1 / d_p + dPhi/ds2, ao[1 + k] = -(dPhi/dv2_k +
// dPhi/dv1_k / d_p)): FMT_AO_Species::set_fundamental_measure_derivatives,
// src/FMT_Species.cpp:667-691; iph = 1/d_p, iph2 = 1/d_p^2. The eta and tensor
// slots are the same for both species.
template <class T, int MODEL>
__device__ __forceinline__ T fmt_phi_point(T* n, T ih, T ih2, T A, T B, T* ao = nullptr, T iph = 0, T iph2 = 0) {
  const T i_pi = (T)(1.0 / 3.14159265358979323846);
  const T i_2pi = (T)(0.5 / 3.14159265358979323846);
  const T i_24pi = (T)(1.0 / (24 * 3.14159265358979323846));
  const T s2 = n[1], s1 = n[1] * ih, s0 = n[1] * ih2;
  const T eta = n[0];
  T v2[3] = {n[2], n[3], n[4]};
  T v1[3] = {n[2] * ih, n[3] * ih, n[4] * ih};
  const T v1_v2 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  const T v2_v2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
  T f1, f2, f3, f1p, f2p, f3p;
  if constexpr (std::is_same<T, dfs>::value) fmt_f_df<MODEL>(eta, f1, f2, f3, f1p, f2p, f3p);
  else fmt_f<T, MODEL>(eta, f1, f2, f3, f1p, f2p, f3p);

  T Phi3, dP3_dS2, dP3_dV2[3], dP3_dT[3][3];
  T Tm[3][3];
  if constexpr (ModelTraits<MODEL>::tensor) {
    Tm[0][0] = n[5]; Tm[0][1] = Tm[1][0] = n[6]; Tm[0][2] = Tm[2][0] = n[7];
    Tm[1][1] = n[8]; Tm[1][2] = Tm[2][1] = n[9]; Tm[2][2] = n[10];
    T vT[3], TT[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) vT[i] = v2[0] * Tm[0][i] + v2[1] * Tm[1][i] + v2[2] * Tm[2][i];
    // T is symmetric, so is T.T: its six distinct entries, mirrored
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i; j < 3; ++j) TT[i][j] = TT[j][i] = Tm[i][0] * Tm[0][j] + Tm[i][1] * Tm[1][j] + Tm[i][2] * Tm[2][j];
    const T vTv = v2[0] * vT[0] + v2[1] * vT[1] + v2[2] * vT[2];
    const T T2 = TT[0][0] + TT[1][1] + TT[2][2];
    // tr(T^3) = sum_ij (T.T)_ij T_ij, the off-diagonal pairs counted twice
    const T T3 = TT[0][0] * Tm[0][0] + TT[1][1] * Tm[1][1] + TT[2][2] * Tm[2][2] +
                 (T)2 * (TT[0][1] * Tm[0][1] + TT[0][2] * Tm[0][2] + TT[1][2] * Tm[1][2]);
    const T a = (MODEL == MODEL_ESFMT) ? A : (T)1, b = (MODEL == MODEL_ESFMT) ? B : (T)-1;
    const T a24 = a * i_24pi, b24 = b * i_24pi;
    Phi3 = a24 * (s2 * s2 * s2 - (T)3 * s2 * v2_v2 + (T)3 * vTv - T3) + b24 * (s2 * s2 * s2 - (T)3 * s2 * T2 + (T)2 * T3);
    dP3_dS2 = a24 * ((T)3 * s2 * s2 - (T)3 * v2_v2) + b24 * ((T)3 * s2 * s2 - (T)3 * T2);
#pragma unroll
    for (int k = 0; k < 3; ++k) dP3_dV2[k] = a24 * (-(T)6 * s2 * v2[k] + (T)3 * vT[k] + (T)3 * vT[k]);
    const T a8 = (T)3 * a24, b4 = (T)6 * b24;  // A/(8 pi), B/(4 pi)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) dP3_dT[j][k] = a8 * (v2[j] * v2[k] - TT[k][j]) + b4 * (-s2 * Tm[k][j] + TT[k][j]);
  } else if constexpr (MODEL == MODEL_RSLT) {
    if (s2 < (T)1e-20) {
      Phi3 = 0; dP3_dS2 = 0; dP3_dV2[0] = dP3_dV2[1] = dP3_dV2[2] = 0;
    } else {
      const T psi = v2_v2 / (s2 * s2);
      const T om = (T)1 - psi;
      Phi3 = (T)(1.0 / (36 * 3.14159265358979323846)) * s2 * s2 * s2 * om * om * om;
      dP3_dS2 = (T)(1.0 / (12 * 3.14159265358979323846)) * s2 * s2 * ((T)1 + psi) * om * om;
#pragma unroll
      for (int k = 0; k < 3; ++k) dP3_dV2[k] = -(T)(1.0 / (6 * 3.14159265358979323846)) * s2 * v2[k] * om * om;
    }
  } else {  // Rosenfeld
    Phi3 = i_24pi * (s2 * s2 * s2 - (T)3 * s2 * v2_v2);
    dP3_dS2 = i_24pi * ((T)3 * s2 * s2 - (T)3 * v2_v2);
#pragma unroll
    for (int k = 0; k < 3; ++k) dP3_dV2[k] = i_24pi * (-(T)6 * s2 * v2[k]);
  }

  T phi = 0;
  phi -= i_pi * s0 * f1;
  phi += i_2pi * (s1 * s2 - v1_v2) * f2;
  phi += Phi3 * f3;

  T d_eta = 0;
  d_eta -= i_pi * s0 * f1p;
  d_eta += i_2pi * (s1 * s2 - v1_v2) * f2p;
  d_eta += Phi3 * f3p;
  const T d_s0 = -i_pi * f1;
  const T d_s1 = i_2pi * s2 * f2;
  T d_s2 = i_2pi * s1 * f2;
  d_s2 += dP3_dS2 * f3;
  n[0] = d_eta;
  n[1] = d_s0 * ih2 + d_s1 * ih + d_s2;
  if (ao) ao[0] = d_s0 * iph2 + d_s1 * iph + d_s2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const T d_v1 = i_2pi * (-v2[k]) * f2;
    T d_v2 = i_2pi * (-v1[k]) * f2;
    d_v2 += dP3_dV2[k] * f3;
    n[2 + k] = -(d_v2 + d_v1 * ih);
    if (ao) ao[1 + k] = -(d_v2 + d_v1 * iph);
  }
  if (ModelTraits<MODEL>::tensor) {
    n[5] = dP3_dT[0][0] * f3;
    n[6] = (T)2 * (dP3_dT[0][1] * f3);
    n[7] = (T)2 * (dP3_dT[0][2] * f3);
    n[8] = dP3_dT[1][1] * f3;
    n[9] = (T)2 * (dP3_dT[1][2] * f3);
    n[10] = dP3_dT[2][2] * f3;
  }
  return phi;
}

// ------------------------------------------------------------ Hessian ---
// Second derivatives of f1, f2, f3 (include/FMT.h: Rosenfeld :163-199, RSLT
// :284-289, WhiteBearI :530-556, WhiteBearII :604-632), the reference's forms.
template <class T, int MODEL>
__device__ __forceinline__ void fmt_fpp(T e, T L, T& f1pp, T& f2pp, T& f3pp) {
  const T one = (T)1;
  const T g = one / (one - e);
  const T g2 = g * g;
  f1pp = -g2;
  f2pp = (T)2 * g2 * g;
  f3pp = (T)6 * g2 * g2;
  if (MODEL == MODEL_RSLT || MODEL == MODEL_WHITEBEAR_I) {
    if (e < (T)1e-12) f3pp = (T)7.5 + (T)28.8 * e;
    else {
      const T ie = one / e, ie2 = ie * ie;
      f3pp = ((T)6 - (T)21 * e + (T)26 * e * e - (T)5 * e * e * e) * ie2 * ie * g2 * g2 + (T)6 * L * ie2 * ie2;
    }
  } else if (MODEL == MODEL_WHITEBEAR_II) {
    if (e < (T)1e-12) {
      f2pp = (T)(20.0 / 9) + (T)7 * e;
      f3pp = (T)7.5 + (T)25.2 * e;
    } else {
      const T ie = one / e, ie2 = ie * ie;
      f2pp = (T)(2.0 / 3.0) * ((T)7 * e * e - (T)5 * e + (T)2) * ie2 * g2 * g + (T)(4.0 / 3.0) * ie2 * ie * L;
      f3pp = -((T)6 - (T)21 * e + (T)26 * e * e - (T)19 * e * e * e + (T)2 * e * e * e * e) * ie2 * ie * g2 * g2 - (T)6 * ie2 * ie2 * L;
    }
  }
}

// sum_b (d2Phi/dn_a dn_b) psi_b for one point (FMT::calculate_d2Phi_dot_V,
// src/FMT.cpp:181-280), in the folded per-species form: n[] are the M weighted
// densities of the state, p[] the M convolutions of v with the same weights
// (FMT::add_second_derivative's Psi, src/FMT.cpp:437-509, with s0 = s/d^2,
// s1 = s/d, v1 = v/d expanded here). On return p[] holds the M fields the
// back-convolution takes: the s slot sums the s0, s1, s2 rows with 1/d^2, 1/d,
// 1; the vector slots carry the conjugated (odd) weights' sign; off-diagonal
// tensor slots sum the (i,j) and (j,i) rows (src/FMT.cpp:530-566).
// pih, pih2: the diameter p[] is read with (1/d, 1/d^2 of its weights): the
// colloid's for the Hessian, the polymer's for the AO force, where p[] holds
// the polymer-weighted convolutions of exp(-Psi) (src/FMT.cpp:393-421).
template <class T, int MODEL>
__device__ __forceinline__ void fmt_d2phi_dot_point(const T* n, T* p, T ih, T ih2, T A, T B, T pih, T pih2) {
  constexpr bool TEN = ModelTraits<MODEL>::tensor;
  const T one = (T)1;
  const T i_pi = (T)(1.0 / 3.14159265358979323846);
  const T i_2pi = (T)(0.5 / 3.14159265358979323846);
  const T i_24pi = (T)(1.0 / (24 * 3.14159265358979323846));
  const T i_8pi = (T)(1.0 / (8 * 3.14159265358979323846));
  const T eta = n[0];
  const T s2 = n[1], s1 = n[1] * ih, s0 = n[1] * ih2;
  T v2[3], v1[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { v2[i] = n[2 + i]; v1[i] = n[2 + i] * ih; }
  T Tm[3][3];
  if (TEN) {
    Tm[0][0] = n[5]; Tm[0][1] = Tm[1][0] = n[6]; Tm[0][2] = Tm[2][0] = n[7];
    Tm[1][1] = n[8]; Tm[1][2] = Tm[2][1] = n[9]; Tm[2][2] = n[10];
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Tm[i][j] = (T)0;
  }
  // Psi in the 19-slot form
  const T Pe = p[0], Ps2 = p[1], Ps1 = p[1] * pih, Ps0 = p[1] * pih2;
  T Pv2[3], Pv1[3], PT[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { Pv2[i] = p[2 + i]; Pv1[i] = p[2 + i] * pih; }
  if (TEN) {
    PT[0][0] = p[5]; PT[0][1] = PT[1][0] = p[6]; PT[0][2] = PT[2][0] = p[7];
    PT[1][1] = p[8]; PT[1][2] = PT[2][1] = p[9]; PT[2][2] = p[10];
  }
  const T v1_v2 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  const T v2_v2 = v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2];
  T f1, f2, f3, f1p, f2p, f3p, f1pp, f2pp, f3pp;
  fmt_f<T, MODEL>(eta, f1, f2, f3, f1p, f2p, f3p);
  fmt_fpp<T, MODEL>(eta, f1, f1pp, f2pp, f3pp);  // f1 = ln(1 - eta)

  // Phi3 and its derivatives
  T Phi3, d_S2, d_V2[3], d_T[3][3], dd_S2S2, dd_V2S2[3], dd_V2V2[3][3], dd_S2T[3][3];
  const T a = (MODEL == MODEL_ESFMT) ? A : one, b = (MODEL == MODEL_ESFMT) ? B : -one;
  if (TEN) {
    T vT[3], TT[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) vT[i] = v2[0] * Tm[0][i] + v2[1] * Tm[1][i] + v2[2] * Tm[2][i];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) TT[i][j] = Tm[i][0] * Tm[0][j] + Tm[i][1] * Tm[1][j] + Tm[i][2] * Tm[2][j];
    const T vTv = v2[0] * vT[0] + v2[1] * vT[1] + v2[2] * vT[2];
    const T T2 = TT[0][0] + TT[1][1] + TT[2][2];
    T T3 = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) T3 += TT[i][j] * Tm[j][i];
    const T a24 = a * i_24pi, b24 = b * i_24pi;
    Phi3 = a24 * (s2 * s2 * s2 - (T)3 * s2 * v2_v2 + (T)3 * vTv - T3) + b24 * (s2 * s2 * s2 - (T)3 * s2 * T2 + (T)2 * T3);
    d_S2 = a24 * ((T)3 * s2 * s2 - (T)3 * v2_v2) + b24 * ((T)3 * s2 * s2 - (T)3 * T2);
#pragma unroll
    for (int k = 0; k < 3; ++k) d_V2[k] = a24 * (-(T)6 * s2 * v2[k] + (T)6 * vT[k]);
    const T a8 = a * i_8pi, b4 = (T)2 * b * i_8pi;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        d_T[j][k] = a8 * (v2[j] * v2[k] - TT[k][j]) + b4 * (-s2 * Tm[k][j] + TT[k][j]);
        dd_S2T[j][k] = b4 * (-Tm[k][j]);
        dd_V2V2[j][k] = a24 * ((T)3 * Tm[j][k] + (T)3 * Tm[k][j] - (j == k ? (T)6 * s2 : (T)0));
      }
    dd_S2S2 = a24 * ((T)6 * s2) + b24 * ((T)6 * s2);
#pragma unroll
    for (int k = 0; k < 3; ++k) dd_V2S2[k] = a24 * (-(T)6 * v2[k]);
  } else if (MODEL == MODEL_RSLT) {
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) { d_T[j][k] = 0; dd_S2T[j][k] = 0; dd_V2V2[j][k] = 0; }
    if (s2 < (T)1e-20) {
      Phi3 = 0; d_S2 = 0; dd_S2S2 = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) { d_V2[k] = 0; dd_V2S2[k] = 0; }
    } else {
      const T is2 = one / s2;
      const T psi = v2_v2 * is2 * is2;
      const T om = one - psi;
      Phi3 = (T)(1.0 / (36 * 3.14159265358979323846)) * s2 * s2 * s2 * om * om * om;
      d_S2 = (T)(1.0 / (12 * 3.14159265358979323846)) * s2 * s2 * (one + psi) * om * om;
      dd_S2S2 = (T)(1.0 / (6 * 3.14159265358979323846)) * s2 * om * (one + psi + (T)2 * psi * psi);
      const T c36 = (T)(1.0 / (36 * 3.14159265358979323846));
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        d_V2[k] = -(T)(1.0 / (6 * 3.14159265358979323846)) * s2 * v2[k] * om * om;
        dd_V2S2[k] = c36 * (-(T)6 * v2[k]) * om * (one + (T)3 * psi);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          dd_V2V2[i][j] = (i == j) ? c36 * (-(T)6 * s2) * om * (om - (T)4 * v2[i] * v2[i] * is2 * is2)
                                   : c36 * ((T)24 * is2) * v2[i] * v2[j] * om;
    }
  } else {  // Rosenfeld
    Phi3 = i_24pi * (s2 * s2 * s2 - (T)3 * s2 * v2_v2);
    d_S2 = i_24pi * ((T)3 * s2 * s2 - (T)3 * v2_v2);
    dd_S2S2 = i_24pi * ((T)6 * s2);
#pragma unroll
    for (int k = 0; k < 3; ++k) { d_V2[k] = i_24pi * (-(T)6 * s2 * v2[k]); dd_V2S2[k] = i_24pi * (-(T)6 * v2[k]); }
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) { d_T[j][k] = 0; dd_S2T[j][k] = 0; dd_V2V2[j][k] = (j == k) ? i_24pi * (-(T)6 * s2) : (T)0; }
  }

  // r = (d2Phi) . Psi, 19 slots
  T Re = (-i_pi * s0 * f1pp + i_2pi * (s1 * s2 - v1_v2) * f2pp + Phi3 * f3pp) * Pe;
  Re += -i_pi * f1p * Ps0;
  const T Rs0 = -i_pi * f1p * Pe;
  Re += i_2pi * s2 * f2p * Ps1;
  T Rs1 = i_2pi * s2 * f2p * Pe;
  const T es2 = i_2pi * s1 * f2p + d_S2 * f3p;
  Re += es2 * Ps2;
  T Rs2 = es2 * Pe;
  T Rv1[3], Rv2[3], RT[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Re += -i_2pi * v2[i] * f2p * Pv1[i];
    Rv1[i] = -i_2pi * v2[i] * f2p * Pe;
    const T ev2 = -i_2pi * v1[i] * f2p + d_V2[i] * f3p;
    Re += ev2 * Pv2[i];
    Rv2[i] = ev2 * Pe;
  }
  Rs1 += i_2pi * f2 * Ps2;
  Rs2 += i_2pi * f2 * Ps1;
  Rs2 += dd_S2S2 * f3 * Ps2;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Rs2 += dd_V2S2[i] * f3 * Pv2[i];
    Rv2[i] += dd_V2S2[i] * f3 * Ps2;
    Rv1[i] += -i_2pi * f2 * Pv2[i];
    Rv2[i] += -i_2pi * f2 * Pv1[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) Rv2[i] += dd_V2V2[i][j] * f3 * Pv2[j];
  }
  if (TEN) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) RT[i][j] = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        Re += d_T[i][j] * f3p * PT[i][j];
        RT[i][j] += d_T[i][j] * f3p * Pe;
        Rs2 += dd_S2T[i][j] * f3 * PT[i][j];
        RT[i][j] += dd_S2T[i][j] * f3 * Ps2;
      }
    // dPhi3/dv2_i dT_jk = A (delta_ij v2_k + delta_ik v2_j) / 8pi
    const T a8 = a * i_8pi;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          T c = 0;
          if (i == j) c += v2[k];
          if (i == k) c += v2[j];
          if (i == j || i == k) {
            Rv2[i] += a8 * c * f3 * PT[j][k];
            RT[j][k] += a8 * c * f3 * Pv2[i];
          }
        }
    // dPhi3/dT_jk dT_lm = [d_lk (-A + 2B) T_mj + d_mj (-A + 2B) T_kl - d_lk d_mj 2B s2] / 8pi
    const T ab = (-a + (T)2 * b) * i_8pi, b2s = -(T)2 * b * s2 * i_8pi;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        T acc = 0;
#pragma unroll
        for (int m = 0; m < 3; ++m) acc += ab * Tm[m][j] * PT[k][m];  // l = k
#pragma unroll
        for (int l = 0; l < 3; ++l) acc += ab * Tm[k][l] * PT[l][j];  // m = j
        acc += b2s * PT[k][j];                                     // l = k, m = j
        RT[j][k] += acc * f3;
      }
  }
  // fold into the M back-convolution fields
  p[0] = Re;
  p[1] = Rs0 * ih2 + Rs1 * ih + Rs2;
#pragma unroll
  for (int i = 0; i < 3; ++i) p[2 + i] = -(Rv1[i] * ih + Rv2[i]);
  if (TEN) {
    p[5] = RT[0][0];
    p[6] = RT[0][1] + RT[1][0];
    p[7] = RT[0][2] + RT[2][0];
    p[8] = RT[1][1];
    p[9] = RT[1][2] + RT[2][1];
    p[10] = RT[2][2];
  }
}

}  // namespace cdft

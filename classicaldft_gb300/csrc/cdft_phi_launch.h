// Launches of the Phi pass, one translation unit per FMT model (cdft_phi_<model>.cu),
// so that the many instances of the pass (precision x model x mode x plan length) compile
// in parallel. The evaluator (cdft_eval.cu) only declares these; each model's unit
// instantiates PhiLauncher<float, MODEL> and PhiLauncher<double, MODEL>.
#pragma once
#include "cdft_kernels_tma.cuh"

namespace cdft {

// Arguments of one Phi-pass launch (T-typed buffers passed untyped; scalars as double).
struct PhiArgs {
  const CUtensorMap* map = nullptr;  // the row-group box map over the M spectra (tensor-copy pass)
  void* Cf = nullptr;                // M spectra, Cx<T>
  Dims d{};
  FFTPlan plan{};                    // the z plan
  const void* tw = nullptr;          // its twiddles, Cx<T>
  double hsd = 1, esA = 1, esB = 0;
  double* part = nullptr;            // block partials of sum Phi
  unsigned* status = nullptr;
  void* NA = nullptr;                // M x N weighted densities, T
  void* XA = nullptr;                // M x N polymer-folded derivative fields, T (AO)
  double iph = 0, iph2 = 0;          // inverse polymer diameter and its square (AO)
};

template <class T, int MODEL>
struct PhiLauncher {
  // Raises the shared-memory limit of the tensor-copy instances for plan length nf to smem
  // and writes their resident blocks per SM to blocks[mode] (kPhiEval, kPhiHess, kPhiStoreN,
  // and kPhiAO when ao).
  static void prepare_tma(int nf, bool ao, size_t smem, int blocks[4]);
  // k_phi_rows_tma<T, MODEL, PhiRowsFor<T, nf>, nf, mode> on grid blocks
  static void launch_tma(int nf, int mode, const PhiArgs& a, int grid, size_t smem, cudaStream_t s);
  // the row kernels of grids the tensor-copy pass does not fit: k_phi_rows (hess = false)
  // and k_hess_rows (hess = true), rb rows per block
  static void prepare_rows(size_t smem);
  static void launch_rows(bool hess, const PhiArgs& a, int rb, unsigned grid, size_t smem, cudaStream_t s);
};

// f(std::integral_constant<int, MODEL>) for a runtime model
template <class F>
inline void with_model(int model, F&& f) {
  switch (model) {
    case MODEL_ROSENFELD: f(std::integral_constant<int, MODEL_ROSENFELD>()); break;
    case MODEL_RSLT: f(std::integral_constant<int, MODEL_RSLT>()); break;
    case MODEL_ESFMT: f(std::integral_constant<int, MODEL_ESFMT>()); break;
    case MODEL_WHITEBEAR_I: f(std::integral_constant<int, MODEL_WHITEBEAR_I>()); break;
    default: f(std::integral_constant<int, MODEL_WHITEBEAR_II>()); break;
  }
}

}  // namespace cdft

// The Phi-pass instances of the Rosenfeld functional, both precisions.
#include "cdft_phi_launch.cuh"

CDFT_PHI_INSTANTIATE(MODEL_ROSENFELD)

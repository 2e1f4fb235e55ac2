// The Phi-pass instances of the White Bear II functional, both precisions.
#include "cdft_phi_launch.cuh"

CDFT_PHI_INSTANTIATE(MODEL_WHITEBEAR_II)

// Types shared by host and device code of the GB300 engine.
#pragma once
#include <cuda_runtime.h>

namespace cdft {

template <class T> struct Cx;
template <> struct Cx<float> { typedef float2 type; };
template <> struct Cx<double> { typedef double2 type; };

constexpr int kMaxStages = 12;
constexpr int kMaxRadix = 32;

// Host-built description of one transform length.
struct FFTPlan {
  int n;
  int nst;
  int radix[kMaxStages];
  int tw_off[kMaxStages];    // offset of the stage's m*p twiddles in the table
  int root_off[kMaxStages];  // offset of the stage's p roots (generic radices)
};

enum Model { MODEL_NONE = -1, MODEL_ROSENFELD = 0, MODEL_RSLT = 1, MODEL_ESFMT = 2, MODEL_WHITEBEAR_I = 3, MODEL_WHITEBEAR_II = 4 };

}  // namespace cdft

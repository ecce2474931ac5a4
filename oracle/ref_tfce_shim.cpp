// ORACLE -- test infrastructure, not product code.
//
// A C-ABI shim around the reference's own TFCE template
// (tfce_mediation/lib/fast_tfce.hpp:11-95), compiled by oracle/build_ref.py
// from the header where it lies in the reference checkout, with its output
// going only to oracle/_ref/.  It lets the tests call the unmodified
// reference sweep on a CSR adjacency without the Cython layer, exactly as
// tfce_mediation/tfce.pyx:44-45 calls it (minT = 0, deltaT = 0).
// <cmath> first: the header calls pow() unqualified and relies on its
// includer for the declaration (the Cython module gets it via Python.h).
#include <cmath>
#include <cstdint>
#include <vector>

#include "fast_tfce.hpp"

extern "C" int ref_tfce(float H, float E, int32_t V, const int64_t* offsets,
                        const int32_t* indices, const float* image, float* enhn) {
  std::vector<std::vector<int> > adj(static_cast<size_t>(V));
  for (int32_t v = 0; v < V; ++v)
    for (int64_t e = offsets[v]; e < offsets[v + 1]; ++e) adj[v].push_back(indices[e]);
  tfce<float>(H, E, 0.0f, 0.0f, adj, image, enhn);
  return 0;
}

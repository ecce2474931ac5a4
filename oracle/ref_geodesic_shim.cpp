// ORACLE -- test infrastructure, not product code.
//
// A C-ABI shim around the reference's own exact geodesic library
// (tfce_mediation/lib/geodesic/, header only), compiled by oracle/build_ref.py
// from the headers where they lie in the reference checkout, with its output
// going only to oracle/_ref/.  It does what
// tfce_mediation/adjacency.pyx:86-106 (compute_distance_parallel) does for
// each source i: propagate from vertex i up to threshold + 1e-10, then ask
// best_source for the distance of every vertex j (j > i when only_greater,
// as the reference lists them; every j != i otherwise) and keep those with
// distance < threshold.
// <cstring> first: the header calls memcpy and relies on its includer for the
// declaration.
#include <cstring>
#include <cstdint>
#include <vector>

#include "geodesic_algorithm_exact.h"

extern "C" int ref_geodesic_lists(int32_t nv, const float* pts, int32_t nf, const int32_t* faces,
                                  double threshold, int32_t only_greater, int32_t src_lo,
                                  int32_t src_hi, int64_t cap, int32_t* out_i, int32_t* out_j,
                                  double* out_d, int64_t* n_out) {
  geodesic::Mesh mesh;
  mesh.initialize_mesh_data<float, int32_t>(static_cast<unsigned>(nv), const_cast<float*>(pts),
                                            static_cast<unsigned>(nf), const_cast<int32_t*>(faces));
  geodesic::GeodesicAlgorithmExact algorithm(&mesh);
  std::vector<geodesic::SurfacePoint> source(1);
  const double max_distance = threshold + 1e-10;  // adjacency.pyx:94
  int64_t n = 0;
  for (int32_t i = src_lo; i < src_hi; ++i) {
    source[0] = geodesic::SurfacePoint(&mesh.vertices()[i]);
    algorithm.propagate(source, max_distance);
    for (int32_t j = only_greater ? i + 1 : 0; j < nv; ++j) {
      if (j == i) continue;
      geodesic::SurfacePoint target(&mesh.vertices()[j]);
      double distance = 0;
      algorithm.best_source(target, distance);
      if (distance < threshold) {
        if (n >= cap) {
          *n_out = n;
          return -4;
        }
        out_i[n] = i;
        out_j[n] = j;
        out_d[n] = distance;
        ++n;
      }
    }
  }
  *n_out = n;
  return 0;
}

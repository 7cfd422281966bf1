// qh_ref_api.cpp — C entry point over the reference's own quickhull
// (wasm/quickhull/QuickHull.cpp, Antti Kuukka, public domain), compiled from
// the reference tree by oracle/Makefile into oracle/_ref/libqh_ref.so.
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle's hull volumes against the
// reference's CPU hull (the one wasm/qh.cpp exposes to src/cpu/hull.ts) and
// serves as the CPU hull of the timed baseline in this container.
#include <cstdint>
#include <cstring>
#include <vector>

#include "quickhull/QuickHull.hpp"

extern "C" int qhref_compute(const double* pts, int n, double eps, double* vOut, int vCap, uint32_t* tOut, int tCap,
                             int* nvOut) {
  quickhull::QuickHull<double> qh;
  auto hull = qh.getConvexHull(pts, (size_t)n, true, false, eps);
  const auto& ib = hull.getIndexBuffer();
  const auto& vb = hull.getVertexBuffer();
  int nv = (int)vb.size(), nt = (int)(ib.size() / 3);
  if (nv > vCap || nt > tCap) return -1;
  for (int i = 0; i < nv; i++) { vOut[3 * i] = vb[i].x; vOut[3 * i + 1] = vb[i].y; vOut[3 * i + 2] = vb[i].z; }
  for (size_t i = 0; i < ib.size(); i++) tOut[i] = (uint32_t)ib[i];
  *nvOut = nv;
  return nt;
}

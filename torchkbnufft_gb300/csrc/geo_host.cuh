// Host-side construction of the per-launch geometry constants.
#pragma once

#include <cmath>

#include "tkbn_common.cuh"

namespace tkbn_host {

// fl(fl(1/K) * fl(2 pi)) — the reference's `2 * np.pi / grid_size` inside
// TorchScript is lowered to reciprocal(K) * 2pi in the working real type
// (torchkbnufft/_nufft/interp.py:171).
template <typename R>
inline R grid_gamma(int64_t K) {
  volatile R r = R(1) / (R)K;
  volatile R twopi = (R)(2.0 * 3.14159265358979323846);
  return r * twopi;
}

template <typename R>
inline tkbn::Geo<R> make_geo(const tkbn_geometry* g, const PointsLayout* L, const void* const* tables,
                             const void* const* dtables) {
  tkbn::Geo<R> geo{};
  geo.ndim = g->ndim;
  geo.ntiles = 1;
  for (int d = 0; d < 3; ++d) {
    const bool on = d < g->ndim;
    geo.K[d] = on ? (int)g->grid_size[d] : 1;
    geo.J[d] = on ? g->numpoints[d] : 1;
    geo.L[d] = on ? g->table_oversamp[d] : 1;
    geo.center[d] = (int)(((int64_t)geo.J[d] * geo.L[d]) / 2);
    geo.tmax[d] = geo.J[d] * geo.L[d];
    geo.T[d] = L ? L->tile[d] : 1;
    geo.P[d] = geo.T[d] + geo.J[d] - 1;
    geo.ntile[d] = L ? L->ntile[d] : 1;
    if (on) geo.ntiles *= geo.ntile[d];
    geo.gam[d] = on ? grid_gamma<R>(g->grid_size[d]) : R(1);
    geo.halfJ[d] = (R)geo.J[d] / R(2);
    geo.Lr[d] = (R)geo.L[d];
    geo.nshift[d] = on ? (R)g->n_shift[d] : R(0);
    geo.tab[d] = (on && tables) ? (const tkbn::cplx<R>*)tables[d] : nullptr;
    geo.half[d] = on && (g->flags & TKBN_TABLES_CONJ_SYMMETRIC) && (((int64_t)geo.J[d] * geo.L[d]) % 2 == 0);
    geo.dtab[d] = (on && dtables) ? (const tkbn::cplx<R>*)dtables[d] : nullptr;
  }
  return geo;
}

}  // namespace tkbn_host

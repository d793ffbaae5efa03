// Map-covariance diagonals with the reference's interface (lib/map_covar.h).
#ifndef DS_GB300_CXX_MAP_COVAR_H
#define DS_GB300_CXX_MAP_COVAR_H

#include <vector>

#include "pcg.h"
#include "pixel.h"
#include "signal_covar.h"

// sigma_m_i = sum_j S_ij^2 / N_j (noise-dominated limit), on the GPU.
void sigma_m_noise_dom(const int n_pix, const NPixel* pixels, const int n_map,
                       const Point* map_coords, const SignalCovarParams* s_params,
                       double* sigma_m);

// sigma_m_i = S_mp[i,:] (S + N)^-1 S_pm[:,i]: one SN-form solve per map point.
class MapCovarDiag {
 public:
  const int n_pix;
  const NPixel* const pixels;
  const int n_map;
  const Point* const map_coords;
  const SignalCovarParams* const s_params;

  MapCovarDiag(const int n_pix, const NPixel* const pixels, const int n_map,
               const Point* const map_coords, const SignalCovarParams* const s_params)
      : n_pix(n_pix), pixels(pixels), n_map(n_map), map_coords(map_coords),
        s_params(s_params) {}

  PCGResult solve_column_pcg(const int i, const PCGParams& pcg_params, double* const x);
  std::vector<PCGResult> solve_pcg(const PCGParams& pcg_params, double* const sigma_m);
};

#endif

/* Layout probe of the C ABI's structs (test infrastructure): prints one line
 * "struct field offset size" per field and "struct - 0 sizeof" per struct,
 * compiled against include/mprw_gpu.h by tests/test_abi.py. */
#include <stddef.h>
#include <stdio.h>

#include "mprw_gpu.h"

#define F(S, f) printf("%s %s %zu %zu\n", #S, #f, offsetof(S, f), sizeof(((S *)0)->f))
#define END(S) printf("%s - 0 %zu\n", #S, sizeof(S))

int main(void) {
  F(mprw_grid_desc, nlay); F(mprw_grid_desc, nrow); F(mprw_grid_desc, ncol); F(mprw_grid_desc, delr);
  F(mprw_grid_desc, delc); F(mprw_grid_desc, top); F(mprw_grid_desc, botm);
  END(mprw_grid_desc);
  F(mprw_options, time_step_kind); F(mprw_options, ts_param); F(mprw_options, advection_kind);
  F(mprw_options, dim_mask); F(mprw_options, dispersion_model); F(mprw_options, stop_weak_sinks);
  F(mprw_options, stop_weak_sources); F(mprw_options, backward); F(mprw_options, stop_zone);
  F(mprw_options, uniform_porosity); F(mprw_options, rng_seed); F(mprw_options, precision);
  END(mprw_options);
  F(mprw_flow_desc, ia); F(mprw_flow_desc, ja); F(mprw_flow_desc, nja); F(mprw_flow_desc, flowja);
  F(mprw_flow_desc, boundary_flows); F(mprw_flow_desc, porosity); F(mprw_flow_desc, retardation);
  F(mprw_flow_desc, iboundts); F(mprw_flow_desc, icboundts); F(mprw_flow_desc, default_icbound);
  F(mprw_flow_desc, heads); F(mprw_flow_desc, celltype); F(mprw_flow_desc, source_flow);
  F(mprw_flow_desc, sink_flow); F(mprw_flow_desc, zones); F(mprw_flow_desc, alpha_l);
  F(mprw_flow_desc, alpha_t); F(mprw_flow_desc, dm_eff); F(mprw_flow_desc, uniform_dispersion);
  F(mprw_flow_desc, steady_state); F(mprw_flow_desc, alpha_lv); F(mprw_flow_desc, alpha_tv);
  END(mprw_flow_desc);
  F(mprw_gpkde_options, origin); F(mprw_gpkde_options, domain_size); F(mprw_gpkde_options, bin_size);
  F(mprw_gpkde_options, n_opt_loops); F(mprw_gpkde_options, min_hover_delta);
  F(mprw_gpkde_options, delta_hover_delta); F(mprw_gpkde_options, max_hover_delta);
  F(mprw_gpkde_options, rel_err_convergence); F(mprw_gpkde_options, skip_error_convergence);
  F(mprw_gpkde_options, unit_volume); F(mprw_gpkde_options, scaling_factor); F(mprw_gpkde_options, precision);
  F(mprw_gpkde_options, isotropic);
  END(mprw_gpkde_options);
  F(mprw_series_options, origin); F(mprw_series_options, domain_size); F(mprw_series_options, bin_size);
  F(mprw_series_options, bin_format); F(mprw_series_options, bin_size_fraction);
  F(mprw_series_options, adapt_grid); F(mprw_series_options, exact_point);
  F(mprw_series_options, effective_weight_format); F(mprw_series_options, initial_smoothing_selection);
  F(mprw_series_options, initial_smoothing_factor); F(mprw_series_options, apply_initial_factor);
  F(mprw_series_options, n_opt_loops); F(mprw_series_options, rel_err_convergence);
  F(mprw_series_options, skip_error_convergence); F(mprw_series_options, only_histogram);
  F(mprw_series_options, compute_raw_density); F(mprw_series_options, unit_volume);
  END(mprw_series_options);
  F(mprw_series_result, n_bins); F(mprw_series_result, delta_bins_origin); F(mprw_series_result, bin_size);
  F(mprw_series_result, grid_origin); F(mprw_series_result, loops_done); F(mprw_series_result, active_bins);
  END(mprw_series_result);
  F(mprw_gpkde_sums, n_active); F(mprw_gpkde_sums, sum_w); F(mprw_gpkde_sums, sum_w2);
  F(mprw_gpkde_sums, sum_dx); F(mprw_gpkde_sums, sum_dx2);
  END(mprw_gpkde_sums);
  F(mprw_adj_options, nzones); F(mprw_adj_options, nsteps); F(mprw_adj_options, checkpoint);
  F(mprw_adj_options, dt); F(mprw_adj_options, velocity_floor); F(mprw_adj_options, seed);
  F(mprw_adj_options, origin); F(mprw_adj_options, bin_size); F(mprw_adj_options, n_bins);
  F(mprw_adj_options, bandwidth);
  END(mprw_adj_options);
  return 0;
}

// hg_plan.h -- host plan math shared by the hdd_ API and the search context.
#pragma once

#include "hella_dedisp.h"

#include <vector>

namespace hg {

std::vector<float> generate_dm_list(double dm_start, double dm_end, double ti_us, double tol,
                                    int nchan, double dt_s, double f0, double df);
std::vector<float> delay_table(int nchan, double dt_s, double f0, double df);
std::vector<int> dm_delays(const std::vector<float> &dms, const std::vector<float> &table);

// Device copies of the plan's delay table and active-channel list.
hdd_error plan_device_tables(hdd_plan p, const int **d_delays, const int **d_chans, int *nact);
// Read-only view of a plan's host tables.
struct PlanView {
  int device;
  void *stream;
  int nchans, ndms, max_delay, nact;
  const int *delays;  // [ndms][nchans]
  const int *chans;   // [nact] active channels
};
PlanView plan_view(hdd_plan p);

// DM tile used for trials [first, first + count) and its largest delay
// spread (cached per range).
int plan_tile(hdd_plan p, int first, int count, int *spread);

}  // namespace hg

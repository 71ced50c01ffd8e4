// hg_search.h -- host helpers shared by the single-beam and batched search
// contexts.
#pragma once

#include "hella_search.h"
#include "hg_internal.h"

#include <vector>

namespace hg {

// Range checks of the search configuration.
hella_status validate_params(const hella_params *p);
// Middle-row smoothing taps of widths width_min << b (b < nbox), each zero
// padded to a multiple of 16: concatenated taps, offsets and padded counts.
void smoothing_taps(const hella_params &p, int nbox, std::vector<float> *taps, std::vector<int> *off,
                    std::vector<int> *n);
// SCRUNCH entries and FLAG1/FLAG2 of the configuration into the flagger state.
void flag_scrunch_params(const hella_params &p, FlagState *f);
// Bytes of one gulp of all beams in the configured input format.
size_t gulp_bytes(const hella_params &p);

}  // namespace hg

// Launch and scheduling defaults of the device carrier loop, chosen by
// phonomc_gb300/autotune.py from timed sweeps on a GB300 (the sweep record it
// writes sits beside it, phonomc_gb300/tuning_record.json). A configuration
// field of 0 selects these values; none of them changes the physics.
// Index [0] is the plain FP64 carrier state, [1] the mixed-precision one.
#pragma once

namespace phmc {
namespace tuning {
// Threads per CTA of the carrier pass (128, 256 or 512).
constexpr int kTransportBlock[2] = {128, 512};
// Resident CTAs per SM of the carrier pass (grid = SMs x this, fewer for
// small populations): sets the carriers each thread walks.
constexpr int kTransportBlocksPerSm[2] = {16, 2};
// Steps between carrier sorts by (mode, cell), or by (cell, mode) in mesh
// domains (0: never), and the smallest population that is sorted at all.
constexpr int kSortInterval[2] = {50, 200};
constexpr double kSortMinCarriers = 2e+06;
// The same for surface-mesh domains (FinFET sweep of the record's "mesh_sorts").
constexpr int kSortIntervalMesh[2] = {25, 25};
// Bin tallies of the carrier pass: 1 sums runs of equal (cell, bin) across
// the lanes of a warp before one FP64 atomic per run, 0 one atomic per carrier.
constexpr int kTallyAggregation[2] = {0, 1};
// Mixed carrier pass: carrier tiles staged in shared memory by bulk
// asynchronous copies one tile ahead (1), or loaded directly (0).
constexpr int kTransportPipeline = 0;
} // namespace tuning
} // namespace phmc

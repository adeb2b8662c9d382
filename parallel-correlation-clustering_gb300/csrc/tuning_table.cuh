// Best-move launch shapes by level-graph size, written by tune_launch.py
// (the fastest launch shape per size class, timed on GB300).
// Columns: max_vertices, group_max_degree, cta_min_degree, grid_waves.
#pragma once

namespace pcc {

constexpr TuningRow kTuningTable[] = {
    {65536u, 32u, 256u, 1.0f},
    {1048576u, 32u, 512u, 2.0f},
    {16777216u, 32u, 512u, 2.0f},
    {4294967295u, 32u, 512u, 2.0f},
};

}  // namespace pcc

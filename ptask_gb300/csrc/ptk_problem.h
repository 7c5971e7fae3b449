// ptk_problem.h -- host-side description of a seeded synthetic FDTD problem, shared by the host
// generator (problem.cpp) and the device-side generator used at request admission (fdtd_batch.cu).
#pragma once

#include <vector>

#include "../../include/ptask_gb300.h"

namespace ptk {

// Axis-aligned dielectric box [lo, hi) in cell coordinates.
struct BoxSpec {
    int lo[3], hi[3];
    float epsr;
};

// Constants, boxes, source node and waveform of problem d (no per-cell arrays).
int problem_plan(const ptk_problem_desc *d, ptk_fdtd_params *p, std::vector<BoxSpec> *boxes, int *si, int *sj,
                 int *sk, std::vector<float> *wave);

}  // namespace ptk

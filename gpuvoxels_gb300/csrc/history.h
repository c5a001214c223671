// The .history text stream of VX3_SimulationManager's simulation loop
// (Voxelyze3/src/VX3/VX3_SimulationManager.cu:40-114): a settings header, then one
// line per recorded step with every surface voxel's pose and deformed corners
// (RecordVoxel) and every link's end positions (RecordLink).
#pragma once
#include <cstdint>
#include <string>

#include "world.h"

namespace gvx {

// Steps between records: int(RecordStepSize / (10000 * recommendedTimeStep * DtFrac)) + 1 (:56).
int history_step_interval(const SimWorld& w, double optimal_dt);

// Header: rescale, material colours, voxel size (:40-50) and the step-interval line (:56-58).
std::string history_header(const SimWorld& w, double optimal_dt);

// One record after loop step `j` (0-based; the reference records when j % interval == 0), at
// simulation time `t` (after the step; `dt` is the step).  d13 = pos3 linMom3 orient4 angMom3 per
// voxel, f4 = temperature and Poisson strains per voxel as the engine holds them after the step
// (the next step's temperature), lsf3 = strain, maxStrain, strainOffset per link.  vflags and
// lflags are the engine's current voxel and link flag words (which voxels are on the surface or
// removed and which links are present, as VX3 detachment and removal change them) and
// local_signal the voxels' VX3 local signals; each may be null (the loaded topology, no signals).
// links4/n_links: the links in use (negative end, positive end, axis, flags) where VX3
// attachment made links during the run (null: the loaded links).
std::string history_record(const SimWorld& w, int64_t j, double t, float dt, const double* d13, const float* f4, const float* lsf3,
                           const int32_t* vflags = nullptr, const int32_t* lflags = nullptr, const double* local_signal = nullptr,
                           const int32_t* links4 = nullptr, int n_links = 0);

}  // namespace gvx

// Host-side simulation model: what a VXA/VXD pair describes, the derived
// material constants, and the voxel/link topology in the reference's order.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "mathtree.h"
#include "xml_dom.h"

namespace gvx {

constexpr int kMaxModelPoints = 16;

// One palette material as parsed (CVXC_Material, Voxelyze3/src/VXA/VX_Object.cpp:1373-1460).
struct PaletteMaterial {
    int model = 0;                 // 0 linear, 1 linear+fail, 2 bilinear, 3 data points
    double E = 0, plastic_mod = 0, yield_stress = 0, fail_stress = 0;
    std::vector<double> strain_data, stress_data;
    double rho = 0, nu = 0, cte = 0, mu_static = 0, mu_kinetic = 0;
    int is_measured = 1;
    std::string name;
    float rgba[4] = {0.5f, 0.5f, 0.5f, 1.0f};   // Display colour (history recorder)
    // VX3 material keys (VXA/VX_Object.cpp:1425-1437): cilia force scale and start time,
    // thermal actuation start time
    double cilia = 0, cilia_on_after = 0, thermal_on_after = 0;
    // VX3 signalling keys (VX_Object.cpp:1420-1424): pacemaker and its period, the factor a
    // relayed signal keeps, the relay delay and the refractory period (seconds)
    int is_pacemaker = 0;
    double pacemaker_period = 0, signal_decay = 0.9, signal_delay = 0.03, inactive_period = 0.03;
    // target voxels (closeness measure, target contacts; VX_Object.cpp:1434) and removal of the
    // material's voxels after a time (SecondaryExperiment, VX_Object.cpp:1427)
    int is_target = 0;
    double remove_after = 0;
    // VX3 Fixed materials: their voxels never move (VX_Object.cpp:1435); Sticky materials'
    // touching voxels may be joined by new links (:1436)
    int fixed = 0;
    int sticky = 0;
};

struct External {
    int voxel = -1;
    int dof_fixed = 0;             // bit0..2 translate xyz, bit3..5 rotate xyz
    float force[3] = {0, 0, 0}, moment[3] = {0, 0, 0};
    double translate[3] = {0, 0, 0}, rotate[3] = {0, 0, 0};
};

// Everything one simulation needs, before any derivation.
struct SimDesc {
    std::string name;
    double vox_size = 0.001;
    double dt_frac = 0.9;
    float gravity_mult = 0;        // CVoxelyze::grav, in g
    bool floor = true;
    bool collisions = true;        // VXA.Simulator.AttachDetach.EnableCollision (VX3 default on)
    float bounding_radius = 0.75f, watch_distance = 1.0f;
    bool temp_enabled = true, vary_temp = false;
    double temp_base = 25, temp_amplitude = 0, temp_period = 0.1;
    int enable_expansion = 0;
    float initial_temp = 0;
    float zeta_internal = 0.1f, zeta_global = 1.0f, zeta_collision = 1.0f;
    bool volume_effects = false;
    std::vector<PaletteMaterial> mats;
    std::vector<int32_t> voxels;   // ix, iy, iz, material (4 per voxel), structure order
    std::vector<double> phase;     // per voxel, in cycles
    std::vector<External> externals;
    MathTree stop_formula, fitness;
    int save_all_positions = 0;
    double max_dist_pairs = 0;     // MaxDistInVoxelLengthsToCountAsPair
    int record_step_size = 0;      // VXA.Simulator.RecordHistory.* (VX3_SimulationManager.cu:344-346)
    int record_voxel = 1, record_link = 0;
    // VX3 extras: cilia (VXA.Simulator.EnableCilia; per-voxel BaseCiliaForce, 3 per voxel, empty
    // when absent) and the force field (VXA.Simulator.ForceField.{x,y,z}_forcefield)
    int enable_cilia = 0;
    std::vector<double> base_cilia;
    MathTree force_field[3];
    bool has_force_field = false;
    // VX3 signals (VXA.Simulator.EnableSignals) and the signal-scaled cilia term (per-voxel
    // ShiftCiliaForce, 3 per voxel, empty when absent)
    int enable_signals = 0;
    std::vector<double> shift_cilia;
    // VX3 link detachment on failure (VXA.Simulator.AttachDetach.EnableDetach) and the
    // secondary experiment (VXA.Simulator.SecondaryExperiment: material removal after a time,
    // initial centre of mass reset after ReinitializeInitialPositionAfterThisManySeconds)
    int enable_detach = 0;
    int secondary_experiment = 0;
    double reinit_initial_after = 0;
    // VX3 attachment (VXA.Simulator.AttachDetach: EnableAttach, SafetyGuard, and the voxel
    // conditions AttachCondition/Condition_0..4; bit k of attach_cond_mask: condition k given)
    int enable_attach = 0;
    int safety_guard = 500;
    MathTree attach_cond[5];
    int attach_cond_mask = 0;
};

// atof of the number field starting at p of a text ending at e (a comma or e ends the
// field); exact same double as atof, faster on plain decimal fields.
double field_atof(const char* p, const char* e);

// Parses a base VXA plus an optional VXD (whose children carrying replace="VXA.a.b"
// replace the subtree at that path, Voxelyze3/src/Utils/ctool.h:49-57).
bool parse_vxa(const std::string& base_xml, const char* vxd_xml, SimDesc* out, std::string* err);
// Applies the VXD rule to a parsed document (exposed for tests).
void merge_vxd(XmlNode* base, const XmlNode& vxd);

// Derived voxel material (CVX_MaterialVoxel after updateDerived), float as in the reference.
struct VoxelMaterial {
    int linear = 1;
    float E = 0, nu = 0, rho = 0, cte = 0, mus = 0, muk = 0, zi = 0, zg = 0, zc = 0, eHat = 0;
    float sigmaYield = -1, sigmaFail = -1, epsYield = -1, epsFail = -1;
    int n = 0;
    float strain[kMaxModelPoints + 2] = {0}, stress[kMaxModelPoints + 2] = {0};
    double nom = 0;
    float grav = 0;
    float mass = 0, massInv = 0, sqrtMass = 0, I = 0, Iinv = 0, c2m = 0, c2i = 0;
    int is_measured = 1;
};
// Derived link material (CVX_MaterialLink): the voxel-material fields plus beam constants.
struct LinkMaterial : VoxelMaterial {
    int vox1 = -1, vox2 = -1;
    float a1 = 0, a2 = 0, b1 = 0, b2 = 0, b3 = 0, sqA1 = 0, sqA2xIp = 0, sqB1 = 0, sqB2xFMp = 0, sqB3xIp = 0;
};

// Topology and constants ready for upload.
struct SimWorld {
    SimDesc desc;
    std::vector<VoxelMaterial> vmats;
    std::vector<LinkMaterial> lmats;
    int nv = 0, nl = 0;
    std::vector<int32_t> link_neg, link_pos;         // voxel indices
    std::vector<uint8_t> link_axis, link_mat;
    std::vector<int32_t> vox_links;                  // 6 per voxel, -1 if absent (direction order X+,X-,Y+,Y-,Z+,Z-)
    std::vector<uint8_t> vox_interior;               // all 6 links present
    std::vector<int32_t> vox_ext;                    // index into desc.externals or -1
    int surface_count = 0;
    std::vector<int32_t> attach_lmat;                // per voxel material: link material of a new link between two of its voxels, or -1
    int loaded_lmats = 0;                            // link materials of the loaded links (attachment's follow them)
};

bool build_world(const SimDesc& d, SimWorld* w, std::string* err);

// Reach masks for the collision exclusion rule (CVX_Voxel::generateNearby,
// Voxelyze3/src/old/VX_Voxel.cpp:394-417): for every voxel, which lattice
// offsets within L1 distance `depth` are reachable through at most `depth`
// links.  One bit per offset of the L1 ball, in the order of l1_ball_offsets().
std::vector<int8_t> l1_ball_offsets(int depth);      // 3 per offset
std::vector<uint32_t> reach_masks(const SimWorld& w, int depth, int words_per_voxel);

}  // namespace gvx

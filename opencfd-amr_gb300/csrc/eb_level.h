// Embedded boundary over a level: device geometry from an implicit function,
// box classes (regular / cut / covered, the test of Source/Advance.cpp:213 and
// :231) and the batched cut-cell stage of the level driver (eb_level.cu).
#pragma once

#include "level.h"

namespace ocfd {

// cut-cell data are stored over grow(bx, EB_GEOM_GROW) in x and y
constexpr int EB_GEOM_GROW = NGR + 1;

struct EbLevel;

// Geometry and classes of every box of L for `eb` (kind OCFD_EB_NONE: none).
// Synchronous; the caller rebuilds the stage tables afterwards.
ocfd_status eb_setup(ocfd_level* L, const ocfd_eb_desc& eb);
void eb_free(ocfd_level* L);
// Stage tables of the cut and covered boxes (stage roles as build_stage_tables).
ocfd_status eb_build_stage_tables(ocfd_level* L, const StageRoles& roles);
// The cut-cell stage s of L: primitives, faces, divergence + RK update (+ CFL).
ocfd_status eb_launch_stage(ocfd_level* L, int s, unsigned flags, cudaStream_t st);
int eb_launches_per_stage(const ocfd_level* L, unsigned flags);
// shared-memory opt-in of the fused cut-cell tile kernel (context creation)
ocfd_status configure_eb_tile();
// true when box b takes the regular path (no body, or classified regular)
bool eb_box_regular(const ocfd_level* L, int b);
// device pointer to the z-invariant volume fraction of box b over grow(bx, 5)
// in x, y (row length gx = nx + 10), or nullptr when the box has no cut cell
// data (regular: all 1, covered: all 0)
const double* eb_box_vfrac(const ocfd_level* L, int b, int* gx);
int eb_box_class(const ocfd_level* L, int b);
// the box's z-invariant flag words over grow(bx, 5) in x, y (nullptr: no data)
const uint32_t* eb_box_flag(const ocfd_level* L, int b);
// views of a cut box's z-invariant geometry (kstride 0): flags, volume
// fraction, area fractions in x, y, z; false when the box has no cut-cell data
bool eb_box_views(const ocfd_level* L, int b, View<const uint32_t>& flag, View<const double>& vfrac,
                  View<const double> ap[3]);

}  // namespace ocfd

// gfs_dropin.h -- plumbing shared by the drop-in PressureSolver, ParticleAdvector
// and CLScalarField: one process-wide libgfs context and conversions between the
// reference's containers (Array3d, MACVelocityField, FluidMaterialGrid) and the
// flat x-fastest arrays of the C ABI (include/gfs.h).
//
// These files replace src/pressuresolver.*, src/particleadvector.* and
// src/clscalarfield.* of a GridFluidSim3D tree; they include that tree's other
// headers and link against libgfs.so.
#ifndef GFS_DROPIN_H
#define GFS_DROPIN_H

#include <cstdint>
#include <string>
#include <vector>

#include "array3d.h"
#include "fluidmaterialgrid.h"
#include "macvelocityfield.h"
#include "vmath.h"

#include "gfs.h"

namespace gfs_dropin {

// The shared context, created on first use on device $GFS_DEVICE (default 0).
// NULL when no CUDA device can be used (gfs_last_error() says why).
gfs_ctx *context();
bool available();
std::string device_name();

// A failed library call: print the library's message and abort, the way the
// reference's OpenCL path reports a failed call (assert on the status).
void check(int status, const char *where);

void to_flat(Array3d<float> *a, std::vector<float> &out);
void from_flat(const std::vector<float> &in, Array3d<float> *a);

struct FlatMAC {
    int ni = 0, nj = 0, nk = 0;
    double dx = 0.0;
    std::vector<float> u, v, w;
};
void mac_to_flat(MACVelocityField *field, FlatMAC &out);

// Material::air / fluid / solid are 0 / 1 / 2 (fluidmaterialgrid.h), the
// codes of the C ABI.
void material_to_flat(FluidMaterialGrid *grid, std::vector<uint8_t> &out);

// std::vector<vmath::vec3> as the C ABI's packed xyz floats.
inline const float *xyz(const std::vector<vmath::vec3> &p) {
    return p.empty() ? nullptr : reinterpret_cast<const float *>(p.data());
}
inline float *xyz(std::vector<vmath::vec3> &p) {
    return p.empty() ? nullptr : reinterpret_cast<float *>(p.data());
}

}  // namespace gfs_dropin

#endif

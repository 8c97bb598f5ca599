// ref_substep_probe.cpp -- TEST INFRASTRUCTURE ONLY (fixture generator probe).
//
// Runs ONE substep of the reference's own FluidSimulation -- fluidsimulation.cpp
// compiled unchanged, with the reference's PressureSolver and the CPU backends
// of oracle/refcpu/ in place of the OpenCL classes -- stage by stage, in the
// order of FluidSimulation::_stepFluid (fluidsimulation.cpp:3262-3360), and
// writes the state after each stage as raw little-endian arrays:
//
//   mat1.u8            material after _updateFluidCells                (stage 1)
//   p1.f32             marker particles (x y z vx vy vz) after stage 1
//   advected.{u,v,w}   _MACVelocity after _advectVelocityField          (stage 5)
//   saved.{u,v,w}      _savedVelocityField after its extrapolation      (stage 5)
//   body.{u,v,w}       _MACVelocity after _applyBodyForcesToVelocityField (stage 6)
//   pressure.f32       the float pressure grid of _updatePressureGrid   (stage 7)
//   applied.{u,v,w}    _MACVelocity after _applyPressureToVelocityField (stage 8)
//   extrap.{u,v,w}     _MACVelocity after _extrapolateFluidVelocities   (stage 9)
//   p11.f32            particles after _updateMarkerParticleVelocities  (stage 11)
//   p12.f32            particles after _advanceRangeOfMarkerParticles over all
//                      particles: RK4 and solid collisions (stage 12 without the
//                      removal pass, so particle q is still input particle q)
//   p12cap.f32         particles after _removeMarkerParticles with srand(seed):
//                      the shuffle and the per-cell cap (fluidsimulation.cpp:3211-3243)
//
// Usage: probe in.state outdir dt gx gy gz max_per_cell shuffle_seed
//
// The probe reaches the private stages by defining private/protected as public
// in its own translation unit, after the standard headers; the library itself is
// compiled unchanged.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <limits>
#include <queue>
#include <sstream>
#include <string>
#include <vector>
#define private public
#define protected public
#include "fluidsimulation.h"
#include "fluidsimulationsavestate.h"
#undef private
#undef protected

static std::string g_dir;

static void put(const std::string &name, const void *data, size_t bytes) {
    std::ofstream f((g_dir + "/" + name).c_str(), std::ios::binary);
    f.write(static_cast<const char *>(data), (std::streamsize)bytes);
}

static void put_grid(const std::string &name, Array3d<float> &a) {
    std::vector<float> v;
    v.reserve((size_t)a.width * a.height * a.depth);
    for (int k = 0; k < a.depth; k++)
        for (int j = 0; j < a.height; j++)
            for (int i = 0; i < a.width; i++) v.push_back(a.get(i, j, k));
    put(name, v.data(), v.size() * sizeof(float));
}

static void put_mac(const std::string &tag, MACVelocityField &f) {
    put_grid(tag + ".u", f._u);
    put_grid(tag + ".v", f._v);
    put_grid(tag + ".w", f._w);
}

static void put_particles(const std::string &name, FluidSimulation &sim) {
    std::vector<float> v;
    v.reserve(sim._markerParticles.size() * 6);
    for (unsigned int q = 0; q < sim._markerParticles.size(); q++) {
        MarkerParticle p = sim._markerParticles[q];
        v.push_back(p.position.x);
        v.push_back(p.position.y);
        v.push_back(p.position.z);
        v.push_back(p.velocity.x);
        v.push_back(p.velocity.y);
        v.push_back(p.velocity.z);
    }
    put(name, v.data(), v.size() * sizeof(float));
}

int main(int argc, char **argv) {
    if (argc < 9) {
        std::fprintf(stderr, "usage: probe in.state outdir dt gx gy gz max_per_cell shuffle_seed\n");
        return 2;
    }
    g_dir = argv[2];
    double dt = std::atof(argv[3]);
    FluidSimulationSaveState state;
    if (!state.loadState(argv[1])) return 3;
    FluidSimulation sim(state);
    state.closeState();
    sim.addBodyForce(std::atof(argv[4]), std::atof(argv[5]), std::atof(argv[6]));
    sim._maxMarkerParticlesPerCell = std::atoi(argv[7]);

    sim._updateFluidCells();
    {
        std::vector<unsigned char> m;
        for (int k = 0; k < sim._ksize; k++)
            for (int j = 0; j < sim._jsize; j++)
                for (int i = 0; i < sim._isize; i++) m.push_back((unsigned char)sim._materialGrid(i, j, k));
        put("mat1.u8", m.data(), m.size());
    }
    put_particles("p1.f32", sim);

    sim._advectVelocityField();
    put_mac("advected", sim._MACVelocity);
    sim._savedVelocityField = sim._MACVelocity;
    sim._extrapolateFluidVelocities(sim._savedVelocityField);
    put_mac("saved", sim._savedVelocityField);

    sim._applyBodyForcesToVelocityField(dt);
    put_mac("body", sim._MACVelocity);

    Array3d<float> pressureGrid(sim._isize, sim._jsize, sim._ksize, 0.0f);
    sim._updatePressureGrid(pressureGrid, dt);
    put_grid("pressure.f32", pressureGrid);
    sim._applyPressureToVelocityField(pressureGrid, dt);
    put_mac("applied", sim._MACVelocity);

    sim._extrapolateFluidVelocities(sim._MACVelocity);
    put_mac("extrap", sim._MACVelocity);

    sim._updateMarkerParticleVelocities();
    put_particles("p11.f32", sim);
    sim._savedVelocityField = MACVelocityField();

    int n = (int)sim._markerParticles.size();
    if (n > 0) sim._advanceRangeOfMarkerParticles(0, n - 1, dt);
    put_particles("p12.f32", sim);

    std::srand((unsigned)std::atoi(argv[8]));
    sim._removeMarkerParticles();
    put_particles("p12cap.f32", sim);
    std::printf("PROBE %d %d %d\n", (int)sim._fluidCellIndices.size(), n, (int)sim._markerParticles.size());
    return 0;
}

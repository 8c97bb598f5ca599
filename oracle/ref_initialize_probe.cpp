// ref_initialize_probe.cpp -- TEST INFRASTRUCTURE ONLY (fixture generator probe).
//
// Seeds a scene with the reference's own FluidSimulation::initialize
// (fluidsimulation.cpp:48-55, 1383-1434), compiled unchanged with the CPU
// backends of oracle/refcpu/, and writes what it made:
//   particles.f32   marker-particle positions (x y z), in creation order
//   mat.u8          the material grid after initialize (i fastest)
// The marker-particle jitter factor is set to 0 (the reference draws the jitter
// from rand(); with 0 the positions are deterministic).
//
// Usage: probe scene.txt outdir
//   scene.txt: "grid ni nj nk dx", then lines "point x y z r",
//   "cuboid x y z w h d" and "solid i j k", in the order to apply them.
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
#undef private
#undef protected

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: probe scene.txt outdir\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::string dir = argv[2], kw;
    int ni = 0, nj = 0, nk = 0;
    double dx = 0.0;
    in >> kw >> ni >> nj >> nk >> dx;
    if (kw != "grid") return 3;
    FluidSimulation sim(ni, nj, nk, dx);
    sim._markerParticleJitterFactor = 0.0;
    while (in >> kw) {
        if (kw == "point") {
            double x, y, z, r;
            in >> x >> y >> z >> r;
            sim.addImplicitFluidPoint(x, y, z, r);
        } else if (kw == "cuboid") {
            double x, y, z, w, h, d;
            in >> x >> y >> z >> w >> h >> d;
            sim.addFluidCuboid(x, y, z, w, h, d);
        } else if (kw == "solid") {
            int i, j, k;
            in >> i >> j >> k;
            std::vector<GridIndex> cells(1, GridIndex(i, j, k));
            sim.addSolidCells(cells);
        } else {
            return 4;
        }
    }
    sim.initialize();
    std::vector<float> p;
    for (unsigned int q = 0; q < sim._markerParticles.size(); q++) {
        MarkerParticle m = sim._markerParticles[q];
        p.push_back(m.position.x);
        p.push_back(m.position.y);
        p.push_back(m.position.z);
    }
    std::ofstream(dir + "/particles.f32", std::ios::binary).write((const char *)p.data(), p.size() * sizeof(float));
    std::vector<unsigned char> m;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) m.push_back((unsigned char)sim._materialGrid(i, j, k));
    std::ofstream(dir + "/mat.u8", std::ios::binary).write((const char *)m.data(), m.size());
    std::printf("PROBE %d\n", (int)sim._markerParticles.size());
    return 0;
}

// particleadvector.cpp -- drop-in ParticleAdvector (see particleadvector.h).
#include "particleadvector.h"

#include <cstdlib>
#include <iostream>

#include "gfs_dropin.h"

ParticleAdvector::ParticleAdvector() {}

// ParticleAdvector::initialize (particleadvector.cpp:33-63): true when the
// accelerator is usable.
bool ParticleAdvector::initialize() {
    _isInitialized = gfs_dropin::available();
    return _isInitialized;
}

void ParticleAdvector::setDevicePreference(std::string devtype) { _devicePreference = devtype; }
void ParticleAdvector::setDevicePreferenceGPU() { _devicePreference = "gpu"; }
void ParticleAdvector::setDevicePreferenceCPU() { _devicePreference = "cpu"; }
void ParticleAdvector::printDeviceInfo() { std::cout << getDeviceInfo() << std::endl; }
std::string ParticleAdvector::getDeviceInfo() { return "CUDA device: " + gfs_dropin::device_name(); }
void ParticleAdvector::printKernelInfo() { std::cout << getKernelInfo() << std::endl; }

std::string ParticleAdvector::getKernelInfo() {
    return "libgfs k_points: one thread per point, separable Catmull-Rom over padded MAC grids (sm_103a)";
}

bool ParticleAdvector::isUsingGPU() { return _isOpenCLEnabled && gfs_dropin::available(); }
bool ParticleAdvector::isUsingCPU() { return false; }
void ParticleAdvector::disableOpenCL() { _isOpenCLEnabled = false; }
void ParticleAdvector::enableOpenCL() { _isOpenCLEnabled = true; }
bool ParticleAdvector::isOpenCLEnabled() { return _isOpenCLEnabled; }
int ParticleAdvector::getKernelWorkLoadSize() { return _kernelWorkLoadSize; }
void ParticleAdvector::setKernelWorkLoadSize(int n) { _kernelWorkLoadSize = n; }

void ParticleAdvector::_requireBackend(const char *where) {
    if (!_isOpenCLEnabled) {
        std::cerr << where << ": the accelerator is disabled (disableOpenCL) and the drop-in has no CPU path"
                  << std::endl;
        std::abort();
    }
    gfs_dropin::check(gfs_dropin::available() ? 0 : GFS_ERR_CUDA, where);
}

void ParticleAdvector::_advect(int order, std::vector<vmath::vec3> &particles, MACVelocityField *vfield,
                               double dt, std::vector<vmath::vec3> &output) {
    _requireBackend("ParticleAdvector::advectParticles");
    gfs_dropin::FlatMAC mac;
    gfs_dropin::mac_to_flat(vfield, mac);
    output.clear();
    output.resize(particles.size());
    gfs_dropin::check(gfs_advect_particles(gfs_dropin::context(), order, mac.ni, mac.nj, mac.nk, mac.dx,
                                           mac.u.data(), mac.v.data(), mac.w.data(), dt,
                                           gfs_dropin::xyz(particles), (int64_t)particles.size(),
                                           gfs_dropin::xyz(output)),
                      "ParticleAdvector::advectParticles");
}

void ParticleAdvector::advectParticlesRK4(std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                                          std::vector<vmath::vec3> &output) {
    _advect(4, particles, vfield, dt, output);
}

void ParticleAdvector::advectParticlesRK3(std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                                          std::vector<vmath::vec3> &output) {
    _advect(3, particles, vfield, dt, output);
}

void ParticleAdvector::advectParticlesRK2(std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                                          std::vector<vmath::vec3> &output) {
    _advect(2, particles, vfield, dt, output);
}

void ParticleAdvector::advectParticlesRK1(std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                                          std::vector<vmath::vec3> &output) {
    _advect(1, particles, vfield, dt, output);
}

void ParticleAdvector::tricubicInterpolate(std::vector<vmath::vec3> &particles, MACVelocityField *vfield,
                                           std::vector<vmath::vec3> &output) {
    _requireBackend("ParticleAdvector::tricubicInterpolate");
    gfs_dropin::FlatMAC mac;
    gfs_dropin::mac_to_flat(vfield, mac);
    output.clear();
    output.resize(particles.size());
    gfs_dropin::check(gfs_tricubic_interpolate(gfs_dropin::context(), mac.ni, mac.nj, mac.nk, mac.dx, mac.u.data(),
                                               mac.v.data(), mac.w.data(), gfs_dropin::xyz(particles),
                                               (int64_t)particles.size(), gfs_dropin::xyz(output)),
                      "ParticleAdvector::tricubicInterpolate");
}

void ParticleAdvector::tricubicInterpolate(std::vector<vmath::vec3> &particles, MACVelocityField *vfield) {
    std::vector<vmath::vec3> output;
    tricubicInterpolate(particles, vfield, output);
    particles.swap(output);
}

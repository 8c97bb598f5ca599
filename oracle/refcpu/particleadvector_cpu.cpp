// particleadvector_cpu.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle).
//
// A CPU backend of the drop-in ParticleAdvector header
// (gridfluidsim3d_gb300/dropin/particleadvector.h) that runs the reference's
// OpenCL-disabled paths: every velocity sample is the reference's own
// MACVelocityField::evaluateVelocityAtPosition (macvelocityfield.cpp:549-559);
// tricubicInterpolate replaces non-finite samples by 0
// (_tricubicInterpolateNoCL / _validateOutput, particleadvector.cpp:1122-1149);
// the RK1..RK4 steps are the formulas of _RK1.._RK4 (:1045-1078) with the same
// float / double casts and the same order of vector operations, applied per
// particle as _advectParticlesRK4NoCL and its siblings do (:1080-1120).
//
// See clscalarfield_cpu.cpp for why this exists.  Nothing in the product links it.
#include <cmath>

#include "particleadvector.h"

namespace {

bool finite3(const vmath::vec3 &v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

// one explicit Runge-Kutta step of the given order from p0
vmath::vec3 rk_step(int order, vmath::vec3 p0, double dt, MACVelocityField *f) {
    vmath::vec3 k1 = f->evaluateVelocityAtPosition(p0);
    if (order == 1) return p0 + (float)dt * k1;
    vmath::vec3 k2 = f->evaluateVelocityAtPosition(p0 + (float)(0.5 * dt) * k1);
    if (order == 2) return p0 + (float)dt * k2;
    if (order == 3) {
        vmath::vec3 k3 = f->evaluateVelocityAtPosition(p0 + (float)(0.75 * dt) * k2);
        return p0 + (float)(dt / 9.0f) * (2.0f * k1 + 3.0f * k2 + 4.0f * k3);
    }
    vmath::vec3 k3 = f->evaluateVelocityAtPosition(p0 + (float)(0.5 * dt) * k2);
    vmath::vec3 k4 = f->evaluateVelocityAtPosition(p0 + (float)dt * k3);
    return p0 + (float)(dt / 6.0f) * (k1 + 2.0f * k2 + 2.0f * k3 + k4);
}

}  // namespace

ParticleAdvector::ParticleAdvector() {}

bool ParticleAdvector::initialize() {
    _isInitialized = true;
    return true;
}

void ParticleAdvector::setDevicePreference(std::string devtype) { _devicePreference = devtype; }
void ParticleAdvector::setDevicePreferenceGPU() { _devicePreference = "gpu"; }
void ParticleAdvector::setDevicePreferenceCPU() { _devicePreference = "cpu"; }
void ParticleAdvector::printDeviceInfo() {}
std::string ParticleAdvector::getDeviceInfo() { return "CPU (the reference's MACVelocityField sampler)"; }
void ParticleAdvector::printKernelInfo() {}
std::string ParticleAdvector::getKernelInfo() { return ""; }
bool ParticleAdvector::isUsingGPU() { return false; }
bool ParticleAdvector::isUsingCPU() { return true; }
void ParticleAdvector::disableOpenCL() { _isOpenCLEnabled = false; }
void ParticleAdvector::enableOpenCL() { _isOpenCLEnabled = true; }
bool ParticleAdvector::isOpenCLEnabled() { return _isOpenCLEnabled; }
int ParticleAdvector::getKernelWorkLoadSize() { return _kernelWorkLoadSize; }
void ParticleAdvector::setKernelWorkLoadSize(int n) { _kernelWorkLoadSize = n; }

void ParticleAdvector::_advect(int order, std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                               std::vector<vmath::vec3> &output) {
    std::vector<vmath::vec3> out;
    out.reserve(particles.size());
    for (size_t q = 0; q < particles.size(); q++) out.push_back(rk_step(order, particles[q], dt, vfield));
    output.swap(out);
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
    if (output.size() < particles.size()) output.resize(particles.size());
    for (size_t q = 0; q < particles.size(); q++) output[q] = vfield->evaluateVelocityAtPosition(particles[q]);
    for (size_t q = 0; q < output.size(); q++)
        if (!finite3(output[q])) output[q] = vmath::vec3(0.0, 0.0, 0.0);
}

void ParticleAdvector::tricubicInterpolate(std::vector<vmath::vec3> &particles, MACVelocityField *vfield) {
    std::vector<vmath::vec3> samples;
    tricubicInterpolate(particles, vfield, samples);
    particles.swap(samples);
}

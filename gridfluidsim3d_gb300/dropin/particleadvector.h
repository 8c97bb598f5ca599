// particleadvector.h -- drop-in replacement of GridFluidSim3D's ParticleAdvector
// (src/particleadvector.h:62-110): the same class and public methods, with the
// tricubic sampling and RK1-4 advection run on the GPU by libgfs
// (gfs_tricubic_interpolate, gfs_advect_particles) instead of OpenCL.
//
// The device toggles are kept.  "OpenCL enabled" (the default) selects the
// CUDA backend; disableOpenCL() leaves no backend (the drop-in has no CPU
// path), and the compute methods then abort with a message.
#ifndef PARTICLEADVECTOR_H
#define PARTICLEADVECTOR_H

#include <vector>
#include <fstream>
#include <algorithm>
#include <string>

#include "macvelocityfield.h"
#include "array3d.h"
#include "grid3d.h"
#include "vmath.h"
#include "fluidsimassert.h"

class ParticleAdvector
{
public:
    ParticleAdvector();

    bool initialize();

    void setDevicePreference(std::string devtype);
    void setDevicePreferenceGPU();
    void setDevicePreferenceCPU();
    void printDeviceInfo();
    std::string getDeviceInfo();
    void printKernelInfo();
    std::string getKernelInfo();
    bool isUsingGPU();
    bool isUsingCPU();
    void disableOpenCL();
    void enableOpenCL();
    bool isOpenCLEnabled();
    int getKernelWorkLoadSize();
    void setKernelWorkLoadSize(int n);

    void advectParticlesRK4(std::vector<vmath::vec3> &particles,
                            MACVelocityField *vfield,
                            double dt,
                            std::vector<vmath::vec3> &output);
    void advectParticlesRK3(std::vector<vmath::vec3> &particles,
                            MACVelocityField *vfield,
                            double dt,
                            std::vector<vmath::vec3> &output);
    void advectParticlesRK2(std::vector<vmath::vec3> &particles,
                            MACVelocityField *vfield,
                            double dt,
                            std::vector<vmath::vec3> &output);
    void advectParticlesRK1(std::vector<vmath::vec3> &particles,
                            MACVelocityField *vfield,
                            double dt,
                            std::vector<vmath::vec3> &output);

    void tricubicInterpolate(std::vector<vmath::vec3> &particles,
                             MACVelocityField *vfield,
                             std::vector<vmath::vec3> &output);

    // method will overwrite particles with output data
    void tricubicInterpolate(std::vector<vmath::vec3> &particles,
                             MACVelocityField *vfield);

private:
    void _advect(int order, std::vector<vmath::vec3> &particles, MACVelocityField *vfield, double dt,
                 std::vector<vmath::vec3> &output);
    void _requireBackend(const char *where);

    bool _isInitialized = false;
    bool _isOpenCLEnabled = true;
    std::string _devicePreference = "gpu";
    int _kernelWorkLoadSize = 10000;
};

#endif

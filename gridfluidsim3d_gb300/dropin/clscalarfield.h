// clscalarfield.h -- drop-in replacement of GridFluidSim3D's CLScalarField
// (src/clscalarfield.h:67-125): the same class and public methods, with the
// point splats run on the GPU by libgfs (gfs_scalar_field_add_point_values)
// instead of OpenCL.  Results are added into the caller's fields, as the
// reference's accelerated path does.
//
// The device toggles are kept.  "OpenCL enabled" (the default) selects the
// CUDA backend; disableOpenCL() leaves no backend (the drop-in has no CPU
// path), and the splat methods then abort with a message.
#ifndef CLSCALARFIELD_H
#define CLSCALARFIELD_H

#include <vector>
#include <fstream>
#include <algorithm>
#include <string>

#include "macvelocityfield.h"
#include "scalarfield.h"
#include "array3d.h"
#include "grid3d.h"
#include "vmath.h"
#include "fluidsimassert.h"

class CLScalarField
{
public:
    CLScalarField();

    bool initialize();
    void addPoints(std::vector<vmath::vec3> &points,
                   double radius,
                   vmath::vec3 offset,
                   double dx,
                   Array3d<float> *field);
    void addPoints(std::vector<vmath::vec3> &points,
                   double radius,
                   vmath::vec3 offset,
                   double dx,
                   ScalarField &field);
    void addPoints(std::vector<vmath::vec3> &points,
                   ScalarField &field);

    void addPointValues(std::vector<vmath::vec3> &points,
                        std::vector<float> &values,
                        double radius,
                        vmath::vec3 offset,
                        double dx,
                        Array3d<float> *field);
    void addPointValues(std::vector<vmath::vec3> &points,
                        std::vector<float> &values,
                        double radius,
                        vmath::vec3 offset,
                        double dx,
                        Array3d<float> *scalarfield,
                        Array3d<float> *weightfield);
    void addPointValues(std::vector<vmath::vec3> &points,
                        std::vector<float> &values,
                        double radius,
                        vmath::vec3 offset,
                        double dx,
                        ScalarField &field);
    void addPointValues(std::vector<vmath::vec3> &points,
                        std::vector<float> &values,
                        ScalarField &field);

    void setMaxScalarFieldValueThreshold(float val);
    void setMaxScalarFieldValueThreshold();
    bool isMaxScalarFieldValueThresholdSet();
    double getMaxScalarFieldValueThreshold();

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

private:
    void _splat(const char *where, std::vector<vmath::vec3> &points, std::vector<float> *values, double radius,
                vmath::vec3 offset, double dx, Array3d<float> *field, Array3d<float> *weightfield);

    bool _isInitialized = false;
    bool _isOpenCLEnabled = true;
    bool _isMaxScalarFieldValueThresholdSet = false;
    float _maxScalarFieldValueThreshold = 1.0;
    std::string _devicePreference = "gpu";
    int _kernelWorkLoadSize = 10000;
};

#endif

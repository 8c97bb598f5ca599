// clscalarfield.cpp -- drop-in CLScalarField (see clscalarfield.h).
#include "clscalarfield.h"

#include <cstdlib>
#include <iostream>

#include "gfs_dropin.h"

CLScalarField::CLScalarField() {}

// CLScalarField::initialize (clscalarfield.cpp:31-66): true when the
// accelerator is usable.
bool CLScalarField::initialize() {
    _isInitialized = gfs_dropin::available();
    return _isInitialized;
}

void CLScalarField::_splat(const char *where, std::vector<vmath::vec3> &points, std::vector<float> *values,
                           double radius, vmath::vec3 offset, double dx, Array3d<float> *field,
                           Array3d<float> *weightfield) {
    if (!_isOpenCLEnabled) {
        std::cerr << where << ": the accelerator is disabled (disableOpenCL) and the drop-in has no CPU path"
                  << std::endl;
        std::abort();
    }
    gfs_dropin::check(gfs_dropin::available() ? 0 : GFS_ERR_CUDA, where);
    if (values != nullptr) {
        FLUIDSIM_ASSERT(points.size() == values->size());
    }
    if (weightfield != nullptr) {
        FLUIDSIM_ASSERT(field->width == weightfield->width && field->height == weightfield->height &&
                        field->depth == weightfield->depth);
    }
    std::vector<float> f, w;
    gfs_dropin::to_flat(field, f);
    if (weightfield != nullptr) gfs_dropin::to_flat(weightfield, w);
    const float off[3] = {offset.x, offset.y, offset.z};
    gfs_dropin::check(gfs_scalar_field_add_point_values(
                          gfs_dropin::context(), gfs_dropin::xyz(points),
                          values != nullptr && !values->empty() ? values->data() : nullptr, (int64_t)points.size(),
                          radius, off, dx, field->width, field->height, field->depth, f.data(),
                          weightfield != nullptr ? w.data() : nullptr, _isMaxScalarFieldValueThresholdSet ? 1 : 0,
                          (double)_maxScalarFieldValueThreshold),
                      where);
    gfs_dropin::from_flat(f, field);
    if (weightfield != nullptr) gfs_dropin::from_flat(w, weightfield);
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, double radius, vmath::vec3 offset, double dx,
                              Array3d<float> *field) {
    _splat("CLScalarField::addPoints", points, nullptr, radius, offset, dx, field, nullptr);
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, double radius, vmath::vec3 offset, double dx,
                              ScalarField &isfield) {
    addPoints(points, radius, offset, dx, isfield.getPointerToScalarField());
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, ScalarField &isfield) {
    addPoints(points, isfield.getPointRadius(), isfield.getOffset(), isfield.getCellSize(),
              isfield.getPointerToScalarField());
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, Array3d<float> *field) {
    _splat("CLScalarField::addPointValues", points, &values, radius, offset, dx, field, nullptr);
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, Array3d<float> *scalarfield,
                                   Array3d<float> *weightfield) {
    _splat("CLScalarField::addPointValues", points, &values, radius, offset, dx, scalarfield, weightfield);
}

// ScalarField overloads (clscalarfield.cpp:269-300): the weight field is used
// when the ScalarField has one enabled
void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, ScalarField &isfield) {
    Array3d<float> *w = isfield.isWeightFieldEnabled() ? isfield.getPointerToWeightField() : nullptr;
    _splat("CLScalarField::addPointValues", points, &values, radius, offset, dx, isfield.getPointerToScalarField(),
           w);
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values,
                                   ScalarField &isfield) {
    addPointValues(points, values, isfield.getPointRadius(), isfield.getOffset(), isfield.getCellSize(), isfield);
}

void CLScalarField::setMaxScalarFieldValueThreshold(float val) {
    _isMaxScalarFieldValueThresholdSet = true;
    _maxScalarFieldValueThreshold = val;
}

void CLScalarField::setMaxScalarFieldValueThreshold() { _isMaxScalarFieldValueThresholdSet = false; }
bool CLScalarField::isMaxScalarFieldValueThresholdSet() { return _isMaxScalarFieldValueThresholdSet; }
double CLScalarField::getMaxScalarFieldValueThreshold() { return _maxScalarFieldValueThreshold; }

void CLScalarField::setDevicePreference(std::string devtype) { _devicePreference = devtype; }
void CLScalarField::setDevicePreferenceGPU() { _devicePreference = "gpu"; }
void CLScalarField::setDevicePreferenceCPU() { _devicePreference = "cpu"; }
void CLScalarField::printDeviceInfo() { std::cout << getDeviceInfo() << std::endl; }
std::string CLScalarField::getDeviceInfo() { return "CUDA device: " + gfs_dropin::device_name(); }
void CLScalarField::printKernelInfo() { std::cout << getKernelInfo() << std::endl; }

std::string CLScalarField::getKernelInfo() {
    return "libgfs k_pt_gather: one thread per node over points sorted by bound corner (sm_103a)";
}

bool CLScalarField::isUsingGPU() { return _isOpenCLEnabled && gfs_dropin::available(); }
bool CLScalarField::isUsingCPU() { return false; }
void CLScalarField::disableOpenCL() { _isOpenCLEnabled = false; }
void CLScalarField::enableOpenCL() { _isOpenCLEnabled = true; }
bool CLScalarField::isOpenCLEnabled() { return _isOpenCLEnabled; }
int CLScalarField::getKernelWorkLoadSize() { return _kernelWorkLoadSize; }
void CLScalarField::setKernelWorkLoadSize(int n) { _kernelWorkLoadSize = n; }

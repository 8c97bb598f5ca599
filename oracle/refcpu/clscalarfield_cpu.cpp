// clscalarfield_cpu.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle).
//
// A CPU backend of the drop-in CLScalarField header
// (gridfluidsim3d_gb300/dropin/clscalarfield.h) that runs the reference's own
// CPU splat, the way the reference's OpenCL-disabled path does
// (CLScalarField::_addPointsNoCL / _addPointValuesNoCL,
// clscalarfield.cpp:1485-1541): the points are splatted into a fresh
// ScalarField of the destination's size with the reference's
// ScalarField::addPoint / addPointValue (scalarfield.cpp:121-201), and the
// result is copied over the destination.
//
// With this file and particleadvector_cpu.cpp in place of the OpenCL classes,
// the reference's fluidsimulation.cpp compiles unchanged and runs its whole CPU
// substep on a machine without OpenCL; oracle/reftree.py builds that library and
// the fixture generators drive it.  Nothing in the product links this file.
//
// Not reproduced: with OpenCL disabled the reference's addPoints(points, radius,
// offset, dx, field) falls through to the accelerated path after the CPU splat
// (no return after _addPointsNoCL, clscalarfield.cpp:75-77).  The substep does not
// call addPoints; the mesher, which does, is not driven by the fixtures.
#include "clscalarfield.h"

namespace {

void overwrite(Array3d<float> *src, Array3d<float> *dst) {
    for (int k = 0; k < dst->depth; k++)
        for (int j = 0; j < dst->height; j++)
            for (int i = 0; i < dst->width; i++) dst->set(i, j, k, src->get(i, j, k));
}

}  // namespace

CLScalarField::CLScalarField() {}

bool CLScalarField::initialize() {
    _isInitialized = true;
    return true;
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, double radius, vmath::vec3 offset, double dx,
                              Array3d<float> *field) {
    ScalarField work(field->width, field->height, field->depth, dx);
    work.setPointRadius(radius);
    work.setOffset(offset);
    for (size_t q = 0; q < points.size(); q++) work.addPoint(points[q]);
    overwrite(work.getPointerToScalarField(), field);
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, double radius, vmath::vec3 offset, double dx,
                              ScalarField &field) {
    addPoints(points, radius, offset, dx, field.getPointerToScalarField());
}

void CLScalarField::addPoints(std::vector<vmath::vec3> &points, ScalarField &field) {
    addPoints(points, field.getPointRadius(), field.getOffset(), field.getCellSize(),
              field.getPointerToScalarField());
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, Array3d<float> *field) {
    ScalarField work(field->width, field->height, field->depth, dx);
    work.setPointRadius(radius);
    work.setOffset(offset);
    for (size_t q = 0; q < points.size(); q++) work.addPointValue(points[q], values[q]);
    overwrite(work.getPointerToScalarField(), field);
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, Array3d<float> *scalarfield,
                                   Array3d<float> *weightfield) {
    ScalarField work(scalarfield->width, scalarfield->height, scalarfield->depth, dx);
    work.enableWeightField();
    work.setPointRadius(radius);
    work.setOffset(offset);
    for (size_t q = 0; q < points.size(); q++) work.addPointValue(points[q], values[q]);
    overwrite(work.getPointerToScalarField(), scalarfield);
    overwrite(work.getPointerToWeightField(), weightfield);
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values, double radius,
                                   vmath::vec3 offset, double dx, ScalarField &field) {
    if (field.isWeightFieldEnabled())
        addPointValues(points, values, radius, offset, dx, field.getPointerToScalarField(),
                       field.getPointerToWeightField());
    else
        addPointValues(points, values, radius, offset, dx, field.getPointerToScalarField());
}

void CLScalarField::addPointValues(std::vector<vmath::vec3> &points, std::vector<float> &values,
                                   ScalarField &field) {
    addPointValues(points, values, field.getPointRadius(), field.getOffset(), field.getCellSize(), field);
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
void CLScalarField::printDeviceInfo() {}
std::string CLScalarField::getDeviceInfo() { return "CPU (the reference's ScalarField splat)"; }
void CLScalarField::printKernelInfo() {}
std::string CLScalarField::getKernelInfo() { return ""; }
bool CLScalarField::isUsingGPU() { return false; }
bool CLScalarField::isUsingCPU() { return true; }
void CLScalarField::disableOpenCL() { _isOpenCLEnabled = false; }
void CLScalarField::enableOpenCL() { _isOpenCLEnabled = true; }
bool CLScalarField::isOpenCLEnabled() { return _isOpenCLEnabled; }
int CLScalarField::getKernelWorkLoadSize() { return _kernelWorkLoadSize; }
void CLScalarField::setKernelWorkLoadSize(int n) { _kernelWorkLoadSize = n; }

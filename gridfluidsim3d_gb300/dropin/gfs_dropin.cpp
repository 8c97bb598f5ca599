// gfs_dropin.cpp -- see gfs_dropin.h.
#include "gfs_dropin.h"

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <mutex>

static_assert(sizeof(vmath::vec3) == 3 * sizeof(float), "vmath::vec3 must be three packed floats");

namespace gfs_dropin {

namespace {
std::mutex g_mutex;
gfs_ctx *g_ctx = nullptr;
bool g_tried = false;
}  // namespace

gfs_ctx *context() {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_tried) {
        g_tried = true;
        const char *dev = std::getenv("GFS_DEVICE");
        int d = dev ? std::atoi(dev) : 0;
        if (gfs_ctx_create(d, &g_ctx) != 0) g_ctx = nullptr;
    }
    return g_ctx;
}

bool available() { return context() != nullptr; }

std::string device_name() {
    gfs_ctx *c = context();
    if (!c) return std::string("no CUDA device: ") + gfs_last_error();
    char buf[256] = {0};
    if (gfs_ctx_device_name(c, buf, (int)sizeof(buf)) != 0) return "unknown";
    return buf;
}

void check(int status, const char *where) {
    if (status == 0) return;
    std::cerr << "libgfs call failed in " << where << " (status " << status << "): " << gfs_last_error()
              << std::endl;
    std::abort();
}

void to_flat(Array3d<float> *a, std::vector<float> &out) {
    out.resize((size_t)a->width * a->height * a->depth);
    size_t q = 0;
    for (int k = 0; k < a->depth; k++)
        for (int j = 0; j < a->height; j++)
            for (int i = 0; i < a->width; i++) out[q++] = a->get(i, j, k);
}

void from_flat(const std::vector<float> &in, Array3d<float> *a) {
    size_t q = 0;
    for (int k = 0; k < a->depth; k++)
        for (int j = 0; j < a->height; j++)
            for (int i = 0; i < a->width; i++) a->set(i, j, k, in[q++]);
}

void mac_to_flat(MACVelocityField *field, FlatMAC &out) {
    field->getGridDimensions(&out.ni, &out.nj, &out.nk);
    out.dx = field->getGridCellSize();
    to_flat(field->getArray3dU(), out.u);
    to_flat(field->getArray3dV(), out.v);
    to_flat(field->getArray3dW(), out.w);
}

void material_to_flat(FluidMaterialGrid *grid, std::vector<uint8_t> &out) {
    out.resize((size_t)grid->width * grid->height * grid->depth);
    size_t q = 0;
    for (int k = 0; k < grid->depth; k++)
        for (int j = 0; j < grid->height; j++)
            for (int i = 0; i < grid->width; i++)
                out[q++] = grid->isCellSolid(i, j, k) ? 2 : (grid->isCellFluid(i, j, k) ? 1 : 0);
}

}  // namespace gfs_dropin

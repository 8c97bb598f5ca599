// savestate.cu -- FluidSimulationSaveState files written from, and read into,
// the device-resident simulation state.
//
// The file format is the reference's (fluidsimulationsavestate.cpp:31-99 writes
// it, :101-150 reads its header), native byte order:
//   int32 i, j, k; double dx; int32 current frame; int32 marker particle count n;
//   int32 diffuse particle count m; int32 solid cell count s; bool (1 byte) brick
//   grid flag; then float32 marker positions [x, y, z] x n; float32 marker
//   velocities x n; float32 diffuse positions x m; diffuse velocities x m;
//   float32 diffuse lifetimes x m; char diffuse types x m; int32 solid cell
//   indices [i, j, k] x s in i-fastest order (:521-573); brick grid data.
//
// The marker particles never pass through a host array of structures: the
// device packs them into xyz triples (the simulation's staging buffers), and the
// triples stream between the device and the file through two pinned chunks, so
// that the copy of one chunk overlaps the file I/O of the other.  Particles are
// written in the device's (cell, id) order and read back with ids 0..n-1 in file
// order, as the reference numbers them by position in _markerParticles.  The
// solid cell list is the material grid's solid cells in the reference's order.
// Diffuse particles and brick grids are outside the simulated core: they are
// written as empty and skipped on reading (their counts are reported).
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gfs_internal.h"

namespace gfs {
namespace {

constexpr size_t kChunkBytes = size_t(32) << 20;   // per pinned staging chunk

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

struct Pinned {
    void *p[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Pinned() {
        for (int b = 0; b < 2; b++) {
            if (p[b]) cudaFreeHost(p[b]);
            if (ev[b]) cudaEventDestroy(ev[b]);
        }
    }
    int init() {
        for (int b = 0; b < 2; b++) {
            GFS_CUDA_CHECK(cudaMallocHost(&p[b], kChunkBytes));
            GFS_CUDA_CHECK(cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming));
        }
        return GFS_OK;
    }
};

struct Header {
    int ni = 0, nj = 0, nk = 0;
    double dx = 0.0;
    int frame = 0, nmarker = 0, ndiffuse = 0, nsolid = 0;
    bool brick = false;
};

bool put(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
bool get(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

// fluidsimulationsavestate.cpp:47-71 (field by field, no padding)
bool put_header(FILE *f, const Header &h) {
    char brick = h.brick ? 1 : 0;
    return put(f, &h.ni, 4) && put(f, &h.nj, 4) && put(f, &h.nk, 4) && put(f, &h.dx, 8) && put(f, &h.frame, 4) &&
           put(f, &h.nmarker, 4) && put(f, &h.ndiffuse, 4) && put(f, &h.nsolid, 4) && put(f, &brick, 1);
}

// fluidsimulationsavestate.cpp:109-117
bool get_header(FILE *f, Header &h) {
    char brick = 0;
    if (!(get(f, &h.ni, 4) && get(f, &h.nj, 4) && get(f, &h.nk, 4) && get(f, &h.dx, 8) && get(f, &h.frame, 4) &&
          get(f, &h.nmarker, 4) && get(f, &h.ndiffuse, 4) && get(f, &h.nsolid, 4) && get(f, &brick, 1)))
        return false;
    h.brick = brick != 0;
    return true;
}

// Device buffer -> file, through the two pinned chunks.
int stream_out(Ctx *ctx, Pinned &pin, const char *dev, size_t bytes, FILE *f, const char *path) {
    cudaStream_t st = ctx->stream;
    size_t nchunks = (bytes + kChunkBytes - 1) / kChunkBytes;
    for (size_t c = 0; c < nchunks + 1; c++) {
        if (c < nchunks) {   // start the copy of chunk c
            size_t off = c * kChunkBytes, n = bytes - off < kChunkBytes ? bytes - off : kChunkBytes;
            GFS_CUDA_CHECK(cudaMemcpyAsync(pin.p[c & 1], dev + off, n, cudaMemcpyDeviceToHost, st));
            GFS_CUDA_CHECK(cudaEventRecord(pin.ev[c & 1], st));
        }
        if (c > 0) {         // write chunk c-1 while chunk c is in flight
            size_t off = (c - 1) * kChunkBytes, n = bytes - off < kChunkBytes ? bytes - off : kChunkBytes;
            GFS_CUDA_CHECK(cudaEventSynchronize(pin.ev[(c - 1) & 1]));
            if (!put(f, pin.p[(c - 1) & 1], n)) {
                cudaStreamSynchronize(st);   // no copy may still target the pinned chunks
                set_error(GFS_ERR_INVALID, "savestate %s: write failed", path);
                return GFS_ERR_INVALID;
            }
        }
    }
    return GFS_OK;
}

// File -> device buffer, through the two pinned chunks.
int stream_in(Ctx *ctx, Pinned &pin, char *dev, size_t bytes, FILE *f, const char *path) {
    cudaStream_t st = ctx->stream;
    size_t nchunks = (bytes + kChunkBytes - 1) / kChunkBytes;
    for (size_t c = 0; c < nchunks; c++) {
        size_t off = c * kChunkBytes, n = bytes - off < kChunkBytes ? bytes - off : kChunkBytes;
        // the chunk's pinned buffer was last used two chunks ago: wait for that copy
        if (c >= 2) GFS_CUDA_CHECK(cudaEventSynchronize(pin.ev[c & 1]));
        if (!get(f, pin.p[c & 1], n)) {
            cudaStreamSynchronize(st);       // no copy may still read the pinned chunks
            set_error(GFS_ERR_INVALID, "savestate %s: file is truncated", path);
            return GFS_ERR_INVALID;
        }
        GFS_CUDA_CHECK(cudaMemcpyAsync(dev + off, pin.p[c & 1], n, cudaMemcpyHostToDevice, st));
        GFS_CUDA_CHECK(cudaEventRecord(pin.ev[c & 1], st));
    }
    GFS_CUDA_CHECK(cudaStreamSynchronize(st));
    return GFS_OK;
}

int open_file(File &fh, const char *path, const char *mode) {
    fh.f = fopen(path, mode);
    if (!fh.f) {
        set_error(GFS_ERR_INVALID, "savestate %s: cannot open (%s)", path, strerror(errno));
        return GFS_ERR_INVALID;
    }
    return GFS_OK;
}

}  // namespace
}  // namespace gfs

using namespace gfs;

extern "C" {

int gfs_savestate_read_header(const char *path, int *ni, int *nj, int *nk, double *dx, int *current_frame,
                              int64_t *num_marker_particles, int64_t *num_diffuse_particles,
                              int64_t *num_solid_cells, int *brick_grid) {
    if (!path) {
        set_error(GFS_ERR_INVALID, "path must not be NULL");
        return GFS_ERR_INVALID;
    }
    File fh;
    int rc = open_file(fh, path, "rb");
    if (rc) return rc;
    Header h;
    if (!get_header(fh.f, h)) {
        set_error(GFS_ERR_INVALID, "savestate %s: header is truncated", path);
        return GFS_ERR_INVALID;
    }
    if (ni) *ni = h.ni;
    if (nj) *nj = h.nj;
    if (nk) *nk = h.nk;
    if (dx) *dx = h.dx;
    if (current_frame) *current_frame = h.frame;
    if (num_marker_particles) *num_marker_particles = h.nmarker;
    if (num_diffuse_particles) *num_diffuse_particles = h.ndiffuse;
    if (num_solid_cells) *num_solid_cells = h.nsolid;
    if (brick_grid) *brick_grid = h.brick ? 1 : 0;
    return GFS_OK;
}

int gfs_sim_save_state(gfs_sim *sim, const char *path, int current_frame) {
    if (!sim || !path) {
        set_error(GFS_ERR_INVALID, "sim and path must not be NULL");
        return GFS_ERR_INVALID;
    }
    Sim *s = &sim->s;
    const int ni = s->g.ni, nj = s->g.nj, nk = s->g.nk;
    // solid cells of the material grid, i fastest (fluidsimulationsavestate.cpp:521-573)
    std::vector<uint8_t> mat((size_t)ni * nj * nk);
    int rc = gfs_sim_get_material(sim, mat.data());
    if (rc) return rc;
    std::vector<int32_t> solid;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (mat[i + (size_t)ni * (j + (size_t)nj * k)] == GFS_SOLID) {
                    solid.push_back(i);
                    solid.push_back(j);
                    solid.push_back(k);
                }
    int64_t n = 0;
    if ((rc = sim_stage_xyz(s, &n))) return rc;
    if (n > INT32_MAX || (int64_t)(solid.size() / 3) > INT32_MAX) {
        set_error(GFS_ERR_INVALID, "savestate %s: counts exceed the format's int32 fields", path);
        return GFS_ERR_INVALID;
    }
    Header h;
    h.ni = ni;
    h.nj = nj;
    h.nk = nk;
    h.dx = s->g.dx;
    h.frame = current_frame;
    h.nmarker = (int)n;
    h.nsolid = (int)(solid.size() / 3);
    File fh;
    if ((rc = open_file(fh, path, "wb"))) return rc;
    Pinned pin;
    if ((rc = pin.init())) return rc;
    if (!put_header(fh.f, h)) {
        set_error(GFS_ERR_INVALID, "savestate %s: write failed", path);
        return GFS_ERR_INVALID;
    }
    const size_t bytes = (size_t)n * 3 * sizeof(float);
    if ((rc = stream_out(s->ctx, pin, s->pos_alt.as<char>(), bytes, fh.f, path))) return rc;
    if ((rc = stream_out(s->ctx, pin, s->vel_alt.as<char>(), bytes, fh.f, path))) return rc;
    // no diffuse particles; the solid cells; no brick grid
    if (!put(fh.f, solid.data(), solid.size() * sizeof(int32_t)) || fclose(fh.f) != 0) {
        fh.f = nullptr;
        set_error(GFS_ERR_INVALID, "savestate %s: write failed", path);
        return GFS_ERR_INVALID;
    }
    fh.f = nullptr;
    return GFS_OK;
}

int gfs_sim_load_state(gfs_sim *sim, const char *path, int *current_frame) {
    if (!sim || !path) {
        set_error(GFS_ERR_INVALID, "sim and path must not be NULL");
        return GFS_ERR_INVALID;
    }
    Sim *s = &sim->s;
    const int ni = s->g.ni, nj = s->g.nj, nk = s->g.nk;
    File fh;
    int rc = open_file(fh, path, "rb");
    if (rc) return rc;
    Header h;
    if (!get_header(fh.f, h)) {
        set_error(GFS_ERR_INVALID, "savestate %s: header is truncated", path);
        return GFS_ERR_INVALID;
    }
    if (h.ni != ni || h.nj != nj || h.nk != nk || h.dx != s->g.dx) {
        set_error(GFS_ERR_INVALID, "savestate %s: grid %d x %d x %d, dx %g does not match the simulation's "
                  "%d x %d x %d, dx %g", path, h.ni, h.nj, h.nk, h.dx, ni, nj, nk, s->g.dx);
        return GFS_ERR_INVALID;
    }
    const long long ncells = (long long)ni * nj * nk;
    if (h.nmarker < 0 || h.nmarker > s->capacity || h.ndiffuse < 0 || h.nsolid < 0 || h.nsolid > ncells) {
        set_error(GFS_ERR_INVALID, "savestate %s: counts (%d marker, %d diffuse, %d solid) outside the "
                  "simulation's capacity %lld and %lld cells", path, h.nmarker, h.ndiffuse, h.nsolid,
                  (long long)s->capacity, ncells);
        return GFS_ERR_INVALID;
    }
    Pinned pin;
    if ((rc = pin.init())) return rc;
    const size_t bytes = (size_t)h.nmarker * 3 * sizeof(float);
    if ((rc = stream_in(s->ctx, pin, s->pos_alt.as<char>(), bytes, fh.f, path))) return rc;
    if ((rc = stream_in(s->ctx, pin, s->vel_alt.as<char>(), bytes, fh.f, path))) return rc;
    // diffuse particles: positions, velocities, lifetimes, types (skipped)
    long long skip = (long long)h.ndiffuse * (3 * 4 + 3 * 4 + 4 + 1);
    if (skip > 0 && fseek(fh.f, (long)skip, SEEK_CUR) != 0) {
        set_error(GFS_ERR_INVALID, "savestate %s: file is truncated", path);
        return GFS_ERR_INVALID;
    }
    // solid cells into an all-air material grid (FluidSimulation::_initializeSolidCellsFromSaveState,
    // fluidsimulation.cpp:1613-1636)
    std::vector<int32_t> idx((size_t)h.nsolid * 3);
    if (!get(fh.f, idx.data(), idx.size() * sizeof(int32_t))) {
        set_error(GFS_ERR_INVALID, "savestate %s: file is truncated", path);
        return GFS_ERR_INVALID;
    }
    std::vector<uint8_t> mat((size_t)ncells, GFS_AIR);
    for (size_t q = 0; q < (size_t)h.nsolid; q++) {
        int i = idx[3 * q], j = idx[3 * q + 1], k = idx[3 * q + 2];
        if (i < 0 || j < 0 || k < 0 || i >= ni || j >= nj || k >= nk) {
            set_error(GFS_ERR_INVALID, "savestate %s: solid cell (%d, %d, %d) outside the grid", path, i, j, k);
            return GFS_ERR_INVALID;
        }
        mat[i + (size_t)ni * (j + (size_t)nj * k)] = GFS_SOLID;
    }
    if ((rc = gfs_sim_set_material(sim, mat.data()))) return rc;
    // marker particles in file order (ids 0..n-1), then sorted as set_particles sorts them
    if ((rc = sim_unstage_xyz(s, h.nmarker))) return rc;
    if (current_frame) *current_frame = h.frame;
    return GFS_OK;
}

}  // extern "C"

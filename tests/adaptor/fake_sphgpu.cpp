// fake_sphgpu.cpp — a host-memory stand-in for libsphgpu, for testing the reference-side adaptor's
// synchronisation logic on a machine without a GPU. TEST INFRASTRUCTURE: it implements the entry points of
// include/sphgpu.h that the adaptor calls, stores every quantity in host memory, and "steps" by a simple
// drift r += v dt (no physics); it counts the uploads and downloads of positions so that a test can check when
// the adaptor moves data. It is compiled only by tests/test_adaptor_cpu.py and never linked into the library.

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "sphgpu.h"

struct sphgpu_handle {
    uint32_t n = 0;
    std::map<std::pair<int, int>, std::vector<unsigned char>> q;
    double dt = 0.;
    // N-body stand-in: index of each particle at the last take_removed, removed indices, merges so far
    std::vector<uint32_t> origin;
    std::vector<uint32_t> removed;
    uint64_t merges = 0;
};

namespace {

int gUploads = 0;
int gDownloads = 0;
int gSteps = 0;

size_t bytesOf(int id, uint64_t n) {
    switch (id) {
    case SPHGPU_Q_POSITION:
    case SPHGPU_Q_ANGULAR_FREQUENCY:
        return 32 * n;
    case SPHGPU_Q_DEVIATORIC_STRESS:
        return 40 * n;
    case SPHGPU_Q_VELOCITY_GRADIENT:
    case SPHGPU_Q_STRAIN_RATE_CORRECTION_TENSOR:
        return 48 * n;
    case SPHGPU_Q_N_FLAWS:
    case SPHGPU_Q_NEIGHBOR_CNT:
    case SPHGPU_Q_FLAG:
    case SPHGPU_Q_MATERIAL_ID:
        return 4 * n;
    default:
        return 8 * n;
    }
}

} // namespace

extern "C" {

void fake_sphgpu_counts(int* uploads, int* downloads, int* steps) {
    *uploads = gUploads;
    *downloads = gDownloads;
    *steps = gSteps;
}

sphgpu_status sphgpu_create(const sphgpu_config* config, sphgpu_handle** out) {
    if (!config || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    *out = new sphgpu_handle();
    (*out)->n = config->particle_count;
    for (uint32_t i = 0; i < config->particle_count; ++i) {
        (*out)->origin.push_back(i);
    }
    (*out)->dt = config->initial_timestep;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_destroy(sphgpu_handle* h) {
    delete h;
    return SPHGPU_OK;
}

const char* sphgpu_last_error(const sphgpu_handle*) {
    return "";
}

sphgpu_status sphgpu_set_quantity(sphgpu_handle* h, int32_t id, int32_t order, const void* src, uint64_t count) {
    if (!h || !src || count != h->n) {
        return SPHGPU_ERR_ARGUMENT;
    }
    auto& v = h->q[{ id, order }];
    v.resize(bytesOf(id, count));
    std::memcpy(v.data(), src, v.size());
    if (id == SPHGPU_Q_POSITION && order == 0) {
        gUploads++;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_get_quantity(sphgpu_handle* h, int32_t id, int32_t order, void* dst, uint64_t count) {
    if (!h || !dst || count != h->n) {
        return SPHGPU_ERR_ARGUMENT;
    }
    auto it = h->q.find({ id, order });
    const size_t bytes = bytesOf(id, count);
    if (it == h->q.end()) {
        std::memset(dst, 0, bytes);
    } else {
        std::memcpy(dst, it->second.data(), bytes);
    }
    if (id == SPHGPU_Q_POSITION && order == 0) {
        gDownloads++;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_integrate(sphgpu_handle* h) {
    return h ? SPHGPU_OK : SPHGPU_ERR_ARGUMENT;
}

sphgpu_status sphgpu_step(sphgpu_handle* h, uint32_t nsteps) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    auto& r = h->q[{ SPHGPU_Q_POSITION, 0 }];
    auto& v = h->q[{ SPHGPU_Q_POSITION, 1 }];
    r.resize(bytesOf(SPHGPU_Q_POSITION, h->n));
    v.resize(bytesOf(SPHGPU_Q_POSITION, h->n));
    double* rp = reinterpret_cast<double*>(r.data());
    const double* vp = reinterpret_cast<const double*>(v.data());
    for (uint32_t s = 0; s < nsteps; ++s) {
        for (uint32_t i = 0; i < h->n; ++i) {
            for (int k = 0; k < 3; ++k) {
                rp[4 * i + k] += vp[4 * i + k] * h->dt;
            }
        }
        gSteps++;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_get_timestep(sphgpu_handle* h, double* dt) {
    *dt = h->dt;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_set_timestep(sphgpu_handle* h, double dt) {
    h->dt = dt;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_phase_times(sphgpu_handle*, double out[SPHGPU_PHASE_COUNT], uint64_t* launches) {
    for (int k = 0; k < SPHGPU_PHASE_COUNT; ++k) {
        out[k] = 0.;
    }
    if (launches) {
        *launches = 0;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_get_pairs(sphgpu_handle*, uint32_t*, uint32_t*, uint64_t, uint64_t* npairs) {
    *npairs = 0;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_build(sphgpu_handle*) {
    return SPHGPU_ERR_UNSUPPORTED;
}

sphgpu_status sphgpu_gravity_eval(sphgpu_handle*, double*, uint64_t) {
    return SPHGPU_ERR_UNSUPPORTED;
}

sphgpu_status sphgpu_gravity_stats(sphgpu_handle*, uint64_t*) {
    return SPHGPU_ERR_UNSUPPORTED;
}

sphgpu_status sphgpu_gravity_eval_points(sphgpu_handle*, const double*, uint64_t, double*) {
    return SPHGPU_ERR_UNSUPPORTED;
}

sphgpu_status sphgpu_gravity_attractors(sphgpu_handle*, const double*, uint64_t, double*, double*, uint64_t) {
    return SPHGPU_ERR_UNSUPPORTED;
}

sphgpu_status sphgpu_get_radius_pairs(sphgpu_handle*, uint32_t*, uint32_t*, uint64_t, uint64_t* npairs) {
    *npairs = 0;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_find_neighbors(sphgpu_handle*, const double*, double, uint32_t*, double*, uint64_t,
    uint64_t* count) {
    *count = 0;
    return SPHGPU_OK;
}

} // extern "C"

extern "C" {

// N-body stand-in: a "collision" merges every odd-indexed particle into its even neighbour (mass added, the
// odd one removed, the order of the others kept), so that a test can check how the adaptor shrinks the Storage
sphgpu_status sphgpu_collide(sphgpu_handle* h, double) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    const uint32_t n = h->n;
    auto compact = [&](int id, int order, size_t bytes) {
        auto it = h->q.find({ id, order });
        if (it == h->q.end()) {
            return;
        }
        std::vector<unsigned char> out;
        for (uint32_t i = 0; i < n; i += 2) {
            out.insert(out.end(), it->second.begin() + i * bytes, it->second.begin() + (i + 1) * bytes);
        }
        it->second = out;
    };
    auto& m = h->q[{ SPHGPU_Q_MASS, 0 }];
    double* mp = reinterpret_cast<double*>(m.data());
    for (uint32_t i = 0; i + 1 < n; i += 2) {
        mp[i] += mp[i + 1];
        h->removed.push_back(h->origin[i + 1]);
        h->merges++;
    }
    std::vector<uint32_t> origin;
    for (uint32_t i = 0; i < n; i += 2) {
        origin.push_back(h->origin[i]);
    }
    h->origin = origin;
    for (int order = 0; order < 3; ++order) {
        compact(SPHGPU_Q_POSITION, order, 32);
    }
    compact(SPHGPU_Q_MASS, 0, 8);
    compact(SPHGPU_Q_ANGULAR_FREQUENCY, 0, 32);
    h->n = (n + 1) / 2;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_take_removed(sphgpu_handle* h, uint32_t* removed, uint64_t capacity, uint64_t* count) {
    *count = h->removed.size();
    if (h->removed.size() > capacity) {
        return SPHGPU_ERR_CAPACITY;
    }
    std::sort(h->removed.begin(), h->removed.end());
    std::copy(h->removed.begin(), h->removed.end(), removed);
    h->removed.clear();
    h->origin.resize(h->n);
    for (uint32_t i = 0; i < h->n; ++i) {
        h->origin[i] = i;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_collision_stats(sphgpu_handle* h, uint64_t out[4]) {
    out[0] = out[1] = h->merges;
    out[2] = out[3] = 0;
    return SPHGPU_OK;
}

} // extern "C"

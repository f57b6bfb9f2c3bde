// extern "C" entry points of libaleator_gb300.so (declared in
// include/aleator_gb300.h). Each call converts exceptions into an
// alea_status and records the message for alea_last_error().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "gcmc.cuh"
#include "grid.cuh"
#include "cif.h"

struct alea_grid {
    alea::GridImpl* impl;
};
struct alea_ewald_state {
    alea::EwaldStateImpl* impl;
};
struct alea_widom {
    alea::WidomImpl* impl;
};
struct alea_gcmc {
    alea::GcmcImpl* impl;
};
struct alea_proposal {
    alea::ProposalImpl* impl;
};
struct alea_grid_batch {
    alea::GridBatchImpl* impl;
};
struct alea_widom_batch {
    alea::WidomBatchImpl* impl;
};

namespace {

thread_local std::string g_last_error;

template <typename F>
alea_status guarded(F&& f) {
    try {
        f();
        g_last_error.clear();
        return ALEA_OK;
    } catch (const alea::Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return ALEA_ERR_RUNTIME;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return ALEA_ERR_RUNTIME;
    } catch (...) {
        g_last_error = "unknown error";
        return ALEA_ERR_RUNTIME;
    }
}

void need(const void* p, const char* what) {
    if (!p) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, std::string(what) + " is NULL");
}

alea_particles particles_or_empty(const alea_particles* p) {
    need(p, "particles");
    return *p;
}

}  // namespace

namespace alea {
void record_last_error(const char* message) { g_last_error = message ? message : ""; }
}  // namespace alea

extern "C" {

const char* alea_status_string(alea_status s) {
    switch (s) {
        case ALEA_OK: return "ok";
        case ALEA_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ALEA_ERR_OUT_OF_RANGE: return "out of range";
        case ALEA_ERR_RUNTIME: return "runtime error";
        case ALEA_ERR_CUDA: return "CUDA error";
        case ALEA_ERR_NO_DEVICE: return "no CUDA device";
        case ALEA_ERR_DEVICE_CHECK: return "device-side check failed";
        default: return "unknown status";
    }
}

size_t alea_last_error(char* buf, size_t cap) {
    if (buf && cap) {
        const size_t n = std::min(cap - 1, g_last_error.size());
        std::memcpy(buf, g_last_error.data(), n);
        buf[n] = '\0';
    }
    return g_last_error.size();
}

alea_status alea_version(int32_t* major, int32_t* minor, int32_t* arch) {
    return guarded([&] {
        if (major) *major = 0;
        if (minor) *minor = 1;
        if (arch) *arch = 103;
    });
}

alea_status alea_device_info(char* name, size_t cap, int32_t* sm_count, int32_t* cc_major,
                             int32_t* cc_minor) {
    return guarded([&] {
        alea::require_device();
        int dev = 0;
        ALEA_CUDA(cudaGetDevice(&dev));
        cudaDeviceProp prop{};
        ALEA_CUDA(cudaGetDeviceProperties(&prop, dev));
        if (name && cap) {
            std::strncpy(name, prop.name, cap - 1);
            name[cap - 1] = '\0';
        }
        if (sm_count) *sm_count = prop.multiProcessorCount;
        if (cc_major) *cc_major = prop.major;
        if (cc_minor) *cc_minor = prop.minor;
    });
}

// ---------------------------------------------------------------- device block cache
alea_status alea_cached_bytes(uint64_t* out) {
    return guarded([&] {
        need(out, "out");
        *out = alea::dev_cached_bytes();
    });
}

alea_status alea_release_cached(uint64_t* freed) {
    return guarded([&] {
        const size_t n = alea::dev_release_cached();
        if (freed) *freed = n;
    });
}

// Fake pointers only: the bookkeeping is checked without touching a device.
alea_status alea_test_block_cache(void) {
    return guarded([&] {
        alea::KeptBlocks kb;
        char a, b, c, d;
        auto fail = [](const char* what) {
            throw alea::Error(ALEA_ERR_RUNTIME, std::string("block cache keying: ") + what);
        };
        const size_t M = 64ull << 20, cap = 4 * M;
        if (!kb.put(0, M, &a, cap) || !kb.put(1, M, &b, cap) || !kb.put(0, 2 * M, &c, cap))
            fail("put under the cap refused");
        if (kb.bytes() != 4 * M) fail("byte count after puts");
        if (kb.put(1, M, &d, cap)) fail("put over the cap accepted");
        if (kb.take(2, M) != nullptr) fail("a block handed to a device that never kept one");
        if (kb.take(1, 2 * M) != nullptr) fail("a block of another device's size handed out");
        if (kb.take(1, M) != &b) fail("device 1's block not returned to device 1");
        if (kb.take(1, M) != nullptr) fail("device 1's block handed out twice");
        if (kb.take(0, M) != &a) fail("device 0's block not returned to device 0");
        if (kb.bytes() != 2 * M) fail("byte count after takes");
        if (!kb.put(1, M, &d, cap)) fail("put after takes refused");
        auto d0 = kb.drain(0);
        if (d0.size() != 1 || d0[0].p != &c || d0[0].device != 0 || d0[0].bytes != 2 * M)
            fail("drain of device 0");
        if (kb.bytes() != M) fail("byte count after a device drain");
        auto rest = kb.drain(-1);
        if (rest.size() != 1 || rest[0].p != &d || rest[0].device != 1) fail("drain of all");
        if (kb.bytes() != 0 || kb.take(1, M) != nullptr) fail("state after the full drain");
    });
}

// ---------------------------------------------------------------- Philox
alea_status alea_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out, uint64_t n) {
    return guarded([&] {
        if (n == 0) return;
        need(ctr, "ctr");
        need(key, "key");
        need(out, "out");
        alea::philox_raw(ctr, key, out, n);
    });
}

alea_status alea_philox_fill_u64(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                 uint64_t* out) {
    return guarded([&] {
        if (n == 0) return;
        need(out, "out");
        alea::require_device();
        alea::DevBuf<uint64_t> d(n);
        alea::philox_fill_u64_device(seed, stream, first, n, d.p, 0);
        d.download(out, n);
        ALEA_CUDA(cudaDeviceSynchronize());
    });
}

alea_status alea_philox_fill_uniform(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                     double* out) {
    return guarded([&] {
        if (n == 0) return;
        need(out, "out");
        alea::require_device();
        alea::DevBuf<double> d(n);
        alea::philox_fill_uniform_device(seed, stream, first, n, d.p, 0);
        d.download(out, n);
        ALEA_CUDA(cudaDeviceSynchronize());
    });
}

alea_status alea_philox_fill_u64_device(uint64_t seed, uint64_t stream_index, uint64_t first,
                                        uint64_t n, uint64_t* out, void* cuda_stream) {
    return guarded([&] {
        if (n) need(out, "out");
        alea::philox_fill_u64_device(seed, stream_index, first, n, out, (cudaStream_t)cuda_stream);
    });
}

alea_status alea_philox_fill_uniform_device(uint64_t seed, uint64_t stream_index, uint64_t first,
                                            uint64_t n, double* out, void* cuda_stream) {
    return guarded([&] {
        if (n) need(out, "out");
        alea::philox_fill_uniform_device(seed, stream_index, first, n, out, (cudaStream_t)cuda_stream);
    });
}

// ---------------------------------------------------------------- grid
alea_status alea_grid_build(const alea_lennard_jones* lj, const alea_particles* framework,
                            const alea_lattice* lattice, const uint32_t* guest_species,
                            uint32_t n_guest, double spacing, int32_t precision, alea_grid** out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(out, "out");
        if (n_guest) need(guest_species, "guest_species");
        *out = nullptr;
        auto* g = new alea_grid{nullptr};
        try {
            g->impl = alea::grid_build(*lj, particles_or_empty(framework), *lattice,
                                       guest_species, n_guest, spacing, precision);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

alea_status alea_grid_build_to_host(const alea_lennard_jones* lj, const alea_particles* framework,
                                    const alea_lattice* lattice, const uint32_t* guest_species,
                                    uint32_t n_guest, double spacing, int32_t precision,
                                    double* const* host_tables, alea_grid** out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(host_tables, "host_tables");
        if (n_guest) need(guest_species, "guest_species");
        for (uint32_t k = 0; k < n_guest; ++k) need(host_tables[k], "host_tables[k]");
        if (out) *out = nullptr;
        alea::GridImpl* impl = alea::grid_build_to_host(*lj, particles_or_empty(framework), *lattice,
                                                        guest_species, n_guest, spacing, precision,
                                                        host_tables);
        if (!out) {
            alea::grid_destroy(impl);
            return;
        }
        *out = new alea_grid{impl};
    });
}

alea_status alea_grid_point_counts(const alea_grid* g, int32_t out[3]) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        alea::grid_counts(g->impl, out);
    });
}

alea_status alea_grid_spacing(const alea_grid* g, double* out) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        *out = alea::grid_spacing(g->impl);
    });
}

alea_status alea_grid_species(const alea_grid* g, uint32_t* out, uint32_t cap, uint32_t* n_out) {
    return guarded([&] {
        need(g, "grid");
        const auto& sp = alea::grid_species(g->impl);
        if (n_out) *n_out = (uint32_t)sp.size();
        for (uint32_t i = 0; out && i < cap && i < sp.size(); ++i) out[i] = sp[i];
    });
}

alea_status alea_grid_interpolate(const alea_grid* g, uint32_t species, const double* xyz,
                                  uint64_t n, double* out) {
    return guarded([&] {
        need(g, "grid");
        if (n) {
            need(xyz, "xyz");
            need(out, "out");
        }
        alea::grid_interpolate_host(g->impl, species, xyz, n, out);
    });
}

alea_status alea_grid_interpolate_device(const alea_grid* g, uint32_t species, const double* xyz,
                                         uint64_t n, double* out, void* cuda_stream) {
    return guarded([&] {
        need(g, "grid");
        alea::grid_interpolate_device(g->impl, species, xyz, n, out, (cudaStream_t)cuda_stream);
    });
}

alea_status alea_grid_download(const alea_grid* g, uint32_t species, double* out, uint64_t n) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        alea::grid_download(g->impl, species, out, n);
    });
}

alea_status alea_grid_table_device(const alea_grid* g, uint32_t species, const double** out) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        *out = alea::grid_table(g->impl, species);
    });
}

alea_status alea_grid_rebuild(alea_grid* g, void* cuda_stream) {
    return guarded([&] {
        need(g, "grid");
        alea::grid_rebuild(g->impl, (cudaStream_t)cuda_stream);
    });
}

alea_status alea_grid_stats_get(const alea_grid* g, alea_grid_stats* out) {
    return guarded([&] {
        need(g, "grid");
        need(out, "out");
        alea::grid_stats(g->impl, out);
    });
}

alea_status alea_grid_serialize(const alea_grid* g, const char* path, const alea_lennard_jones* lj,
                                const alea_particles* framework, const alea_lattice* lattice,
                                const uint32_t* guest_species, uint32_t n_guest) {
    return guarded([&] {
        need(g, "grid");
        need(path, "path");
        need(lj, "lj");
        need(lattice, "lattice");
        const auto& sp = alea::grid_species(g->impl);
        int32_t counts[3];
        alea::grid_counts(g->impl, counts);
        const uint64_t nodes = (uint64_t)counts[0] * counts[1] * counts[2];
        std::vector<std::vector<double>> tables(sp.size(), std::vector<double>(nodes));
        for (size_t i = 0; i < sp.size(); ++i) alea::grid_download(g->impl, sp[i], tables[i].data(), nodes);
        alea::grid_cache_write(path, *lj, particles_or_empty(framework), *lattice, guest_species,
                               n_guest, alea::grid_spacing(g->impl), counts, sp, tables);
    });
}

alea_status alea_grid_cache_file_name(const alea_lennard_jones* lj, const alea_particles* framework,
                                      const alea_lattice* lattice, const uint32_t* guest_species,
                                      uint32_t n_guest, double spacing, char* out, size_t cap) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(out, "out");
        const std::string s = alea::grid_cache_file_name(*lj, particles_or_empty(framework),
                                                         *lattice, guest_species, n_guest, spacing);
        if (s.size() + 1 > cap)
            throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "alea_grid_cache_file_name: buffer too small");
        std::memcpy(out, s.c_str(), s.size() + 1);
    });
}

struct alea_structure {
    alea::Structure s;
};

alea_status alea_read_cif(const char* path, alea_structure** out) {
    return guarded([&] {
        need(path, "path");
        need(out, "out");
        *out = nullptr;
        auto* h = new alea_structure{alea::read_cif(path)};
        *out = h;
    });
}

alea_status alea_structure_sizes(const alea_structure* s, uint64_t* n_atoms, uint32_t* n_species) {
    return guarded([&] {
        need(s, "structure");
        if (n_atoms) *n_atoms = s->s.x.size();
        if (n_species) *n_species = (uint32_t)s->s.symbols.size();
    });
}

alea_status alea_structure_lattice(const alea_structure* s, double m[9]) {
    return guarded([&] {
        need(s, "structure");
        need(m, "m");
        std::memcpy(m, s->s.m, sizeof s->s.m);
    });
}

alea_status alea_structure_atoms(const alea_structure* s, double* x, double* y, double* z,
                                 double* charge, double* mass, uint32_t* species,
                                 double* occupancy) {
    return guarded([&] {
        need(s, "structure");
        const alea::Structure& t = s->s;
        const size_t n = t.x.size();
        auto put = [n](auto* dst, const auto& src) {
            if (dst && n) std::memcpy(dst, src.data(), n * sizeof(src[0]));
        };
        put(x, t.x);
        put(y, t.y);
        put(z, t.z);
        put(charge, t.charge);
        put(mass, t.mass);
        put(species, t.species);
        put(occupancy, t.occupancy);
    });
}

static void copy_text(const std::string& v, char* out, size_t cap, const char* who) {
    if (v.size() + 1 > cap)
        throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, std::string(who) + ": buffer too small");
    std::memcpy(out, v.c_str(), v.size() + 1);
}

alea_status alea_structure_species_symbol(const alea_structure* s, uint32_t species, char* out,
                                          size_t cap) {
    return guarded([&] {
        need(s, "structure");
        need(out, "out");
        if (species >= s->s.symbols.size())
            throw alea::Error(ALEA_ERR_OUT_OF_RANGE, "alea_structure_species_symbol: species out of range");
        copy_text(s->s.symbols[species], out, cap, "alea_structure_species_symbol");
    });
}

alea_status alea_structure_source_label(const alea_structure* s, uint64_t atom, char* out,
                                        size_t cap) {
    return guarded([&] {
        need(s, "structure");
        need(out, "out");
        if (atom >= s->s.labels.size())
            throw alea::Error(ALEA_ERR_OUT_OF_RANGE, "alea_structure_source_label: atom out of range");
        copy_text(s->s.labels[atom], out, cap, "alea_structure_source_label");
    });
}

alea_status alea_structure_destroy(alea_structure* s) {
    return guarded([&] { delete s; });
}

alea_status alea_test_grid_tile_wait_limit(int64_t limit) {
    return guarded([&] { alea::grid_test_set_tile_wait_limit(limit); });
}

alea_status alea_grid_cache_hit(const char* cache_dir, const alea_lennard_jones* lj,
                                const alea_particles* framework, const alea_lattice* lattice,
                                const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                int32_t* hit) {
    return guarded([&] {
        need(cache_dir, "cache_dir");
        need(lj, "lj");
        need(lattice, "lattice");
        need(hit, "hit");
        if (n_guest) need(guest_species, "guest_species");
        *hit = alea::grid_cache_hit(cache_dir, *lj, particles_or_empty(framework), *lattice,
                                    guest_species, n_guest, spacing)
                   ? 1
                   : 0;
    });
}

alea_status alea_grid_load_cache(const char* cache_dir, const alea_lennard_jones* lj,
                                 const alea_particles* framework, const alea_lattice* lattice,
                                 const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                 alea_grid** out) {
    return guarded([&] {
        need(cache_dir, "cache_dir");
        need(lj, "lj");
        need(lattice, "lattice");
        need(out, "out");
        *out = nullptr;
        int32_t counts[3];
        std::vector<uint32_t> sp;
        std::vector<std::vector<double>> tables;
        if (!alea::grid_cache_read(cache_dir, *lj, particles_or_empty(framework), *lattice,
                                   guest_species, n_guest, spacing, counts, sp, tables))
            return;
        auto* g = new alea_grid{nullptr};
        try {
            g->impl = alea::grid_from_tables(*lattice, spacing, counts, sp, tables);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

alea_status alea_grid_destroy(alea_grid* g) {
    return guarded([&] {
        if (!g) return;
        alea::grid_destroy(g->impl);
        delete g;
    });
}

// ---------------------------------------------------------------- Lennard-Jones
alea_status alea_lj_particle_energy(const alea_lennard_jones* lj, const alea_particles* particles,
                                    const alea_lattice* lattice, const uint64_t* query,
                                    uint64_t n_query, const uint64_t* excluded, uint64_t n_excluded,
                                    double* out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        if (n_query) {
            need(query, "query");
            need(out, "out");
        }
        if (n_excluded) need(excluded, "excluded");
        alea::lj_particle_energy(*lj, particles_or_empty(particles), *lattice, query, n_query,
                                 excluded, n_excluded, out);
    });
}

// LennardJones::tailEnergyCorrection (lennard_jones.cc:217-257): an
// O(species^2) host formula over the species counts.
alea_status alea_lj_tail_correction(const alea_lennard_jones* lj, const alea_particles* particles,
                                    const alea_lattice* lattice, double* out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(out, "out");
        const alea_particles p = particles_or_empty(particles);
        const alea::Lattice L = alea::make_lattice(lattice->m);
        const double volume = std::fabs(L.volume);
        const double rc = lj->cutoff;
        std::vector<uint64_t> counts(lj->n_species, 0);
        for (uint64_t i = 0; i < p.n; ++i) {
            const uint32_t s = p.species ? p.species[i] : 0u;
            if (s >= lj->n_species)
                throw alea::Error(ALEA_ERR_OUT_OF_RANGE, "tailEnergyCorrection: species out of range");
            counts[s] += 1;
        }
        std::vector<alea::PairParams> table((size_t)lj->n_species * lj->n_species);
        alea::mixed_table(*lj, table.data());
        double total = 0.0;
        for (uint32_t a = 0; a < lj->n_species; ++a) {
            if (!counts[a]) continue;
            for (uint32_t b = 0; b < lj->n_species; ++b) {
                if (!counts[b]) continue;
                const alea::PairParams& pp = table[(size_t)a * lj->n_species + b];
                const double sr3 = pp.sigma * pp.sigma * pp.sigma;
                const double sr9 = sr3 * sr3 * sr3 / (rc * rc * rc * rc * rc * rc * rc * rc * rc);
                const double sr3rc3 = sr3 / (rc * rc * rc);
                total += (double)counts[a] * (double)counts[b] *
                         (pp.eps * sr3 * ((4.0 / 9.0) * sr9 - (4.0 / 3.0) * sr3rc3));
            }
        }
        *out = (2.0 * alea::kPi / volume) * total;
    });
}

// ---------------------------------------------------------------- Ewald
alea_status alea_ewald_reciprocal_terms(const alea_lattice* lattice, double alpha, int32_t kmax,
                                        double* k, double* weight, uint64_t cap, uint64_t* n_out) {
    return guarded([&] {
        need(lattice, "lattice");
        if (!(alpha > 0.0)) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "Ewald: alpha must be positive");
        if (kmax < 1) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "Ewald: kMax must be at least 1");
        const alea::Lattice L = alea::make_lattice(lattice->m);
        const uint64_t n = alea::ewald_terms_host(L, alpha, kmax, k, weight, nullptr, (k || weight) ? cap : 0);
        if (n_out) *n_out = n;
    });
}

alea_status alea_ewald_real_space_particle_energy(const alea_ewald* ewald,
                                                  const alea_particles* particles,
                                                  const alea_lattice* lattice,
                                                  const uint64_t* query, uint64_t n_query,
                                                  const uint64_t* excluded, uint64_t n_excluded,
                                                  double* out) {
    return guarded([&] {
        need(ewald, "ewald");
        need(lattice, "lattice");
        if (n_query) {
            need(query, "query");
            need(out, "out");
        }
        if (n_excluded) need(excluded, "excluded");
        alea::ewald_real_space_particle_energy(*ewald, particles_or_empty(particles), *lattice, query,
                                               n_query, excluded, n_excluded, out);
    });
}

alea_status alea_ewald_energy_breakdown(const alea_ewald* ewald, const alea_particles* particles,
                                        const alea_lattice* lattice, const uint64_t* exclusions,
                                        uint64_t n_exclusions, double out[5]) {
    return guarded([&] {
        need(ewald, "ewald");
        need(lattice, "lattice");
        need(out, "out");
        if (n_exclusions) need(exclusions, "exclusions");
        alea::ewald_breakdown(*ewald, particles_or_empty(particles), *lattice, exclusions,
                              n_exclusions, out);
    });
}

alea_status alea_ewald_state_create(const alea_ewald* ewald, const alea_particles* particles,
                                    const alea_lattice* lattice, alea_ewald_state** out) {
    return guarded([&] {
        need(ewald, "ewald");
        need(lattice, "lattice");
        need(out, "out");
        *out = nullptr;
        auto* s = new alea_ewald_state{nullptr};
        try {
            s->impl = alea::ewald_state_create(*ewald, particles_or_empty(particles), *lattice);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}

alea_status alea_ewald_state_committed_energy(const alea_ewald_state* s, double* out) {
    return guarded([&] {
        need(s, "state");
        need(out, "out");
        *out = alea::ewald_state_energy(s->impl);
    });
}

alea_status alea_ewald_state_propose(const alea_ewald_state* s, const double* removed,
                                     uint64_t n_removed, const double* added, uint64_t n_added,
                                     double* delta) {
    return guarded([&] {
        need(s, "state");
        need(delta, "delta");
        if (n_removed) need(removed, "removed");
        if (n_added) need(added, "added");
        *delta = alea::ewald_state_propose(s->impl, removed, n_removed, added, n_added);
    });
}

alea_status alea_ewald_state_commit(alea_ewald_state* s, const double* removed, uint64_t n_removed,
                                    const double* added, uint64_t n_added) {
    return guarded([&] {
        need(s, "state");
        if (n_removed) need(removed, "removed");
        if (n_added) need(added, "added");
        alea::ewald_state_commit(s->impl, removed, n_removed, added, n_added);
    });
}

alea_status alea_ewald_state_recompute(const alea_ewald_state* s, const alea_particles* particles,
                                       uint64_t n_molecules, const uint64_t* offsets,
                                       const uint64_t* indices, double* out) {
    return guarded([&] {
        need(s, "state");
        need(out, "out");
        if (n_molecules) {
            need(offsets, "offsets");
            need(indices, "indices");
        }
        *out = alea::ewald_state_recompute(s->impl, particles_or_empty(particles), n_molecules,
                                           offsets, indices);
    });
}

alea_status alea_ewald_state_resync(alea_ewald_state* s, const alea_particles* particles,
                                    uint64_t n_molecules, const uint64_t* offsets,
                                    const uint64_t* indices) {
    return guarded([&] {
        need(s, "state");
        if (n_molecules) {
            need(offsets, "offsets");
            need(indices, "indices");
        }
        alea::ewald_state_resync(s->impl, particles_or_empty(particles), n_molecules, offsets,
                                 indices);
    });
}

alea_status alea_ewald_state_raw(const alea_ewald_state* s, double* out, uint64_t cap,
                                 uint64_t* n_out) {
    return guarded([&] {
        need(s, "state");
        const auto raw = alea::ewald_state_raw(s->impl);
        if (n_out) *n_out = raw.size();
        for (uint64_t i = 0; out && i < cap && i < raw.size(); ++i) out[i] = raw[i];
    });
}

alea_status alea_ewald_state_term_count(const alea_ewald_state* s, uint64_t* out) {
    return guarded([&] {
        need(s, "state");
        need(out, "out");
        *out = alea::ewald_state_nk(s->impl);
    });
}

alea_status alea_ewald_state_destroy(alea_ewald_state* s) {
    return guarded([&] {
        if (!s) return;
        alea::ewald_state_destroy(s->impl);
        delete s;
    });
}

// ---------------------------------------------------------------- Widom
alea_status alea_widom_create(const alea_lennard_jones* lj, const alea_ewald* ewald,
                              const alea_particles* framework, const alea_lattice* lattice,
                              const alea_molecule_species* guest, double temperature,
                              int32_t precision, alea_widom** out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(guest, "guest");
        need(out, "out");
        *out = nullptr;
        auto* w = new alea_widom{nullptr};
        try {
            w->impl = alea::widom_create(*lj, ewald, particles_or_empty(framework), *lattice, *guest,
                                         temperature, precision);
        } catch (...) {
            delete w;
            throw;
        }
        *out = w;
    });
}

alea_status alea_widom_run(alea_widom* w, uint64_t seed, uint64_t stream, uint64_t first_trial,
                           uint64_t n_trials, int32_t draw_order, alea_widom_result* out,
                           double* per_trial_du) {
    return guarded([&] {
        need(w, "widom");
        need(out, "out");
        alea::widom_run(w->impl, seed, stream, first_trial, n_trials, draw_order, out, per_trial_du);
    });
}

alea_status alea_widom_samples(alea_widom* w, const alea_proposal* proposal, uint64_t seed,
                               uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                               int32_t draw_order, float* samples_device) {
    return guarded([&] {
        need(w, "widom");
        alea::require(samples_device || n_trials == 0, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_widom_samples: samples_device is required");
        if (proposal) {
            const alea::ProposalTable t = alea::proposal_table(proposal->impl);
            alea::widom_samples(w->impl, seed, stream, first_trial, n_trials, draw_order,
                                samples_device, &t);
        } else {
            alea::widom_samples(w->impl, seed, stream, first_trial, n_trials, draw_order,
                                samples_device, nullptr);
        }
    });
}

alea_status alea_widom_run_biased(alea_widom* w, const alea_proposal* p, uint64_t seed,
                                  uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                                  alea_widom_result* out, double* per_trial_du,
                                  double* per_trial_frac) {
    return guarded([&] {
        need(w, "widom");
        need(p, "proposal");
        need(out, "out");
        const alea::ProposalTable t = alea::proposal_table(p->impl);
        alea::widom_run(w->impl, seed, stream, first_trial, n_trials, ALEA_DRAWS_RIGHT_TO_LEFT, out,
                        per_trial_du, &t, per_trial_frac);
    });
}

alea_status alea_grid_batch_create(uint32_t n, const alea_lennard_jones* lj,
                                   const alea_particles* frameworks, const alea_lattice* lattices,
                                   const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                   alea_grid_batch** out) {
    return guarded([&] {
        need(out, "out");
        *out = nullptr;
        alea::require(lj && frameworks && lattices && guest_species, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_grid_batch_create: lj, frameworks, lattices and guest_species are required");
        auto* impl = alea::grid_batch_create(n, lj, frameworks, lattices, guest_species, n_guest,
                                             spacing);
        *out = new alea_grid_batch{impl};
    });
}

alea_status alea_grid_batch_build(alea_grid_batch* b, void* cuda_stream) {
    return guarded([&] {
        need(b, "grid batch");
        alea::grid_batch_build(b->impl, (cudaStream_t)cuda_stream);
    });
}

alea_status alea_grid_batch_stats_get(const alea_grid_batch* b, alea_grid_batch_stats* out) {
    return guarded([&] {
        need(b, "grid batch");
        need(out, "out");
        alea::grid_batch_stats(b->impl, out);
    });
}

alea_status alea_grid_batch_point_counts(const alea_grid_batch* b, uint32_t grid, int32_t out[3]) {
    return guarded([&] {
        need(b, "grid batch");
        need(out, "out");
        alea::grid_counts(alea::grid_batch_item(b->impl, grid), out);
    });
}

alea_status alea_grid_batch_download(const alea_grid_batch* b, uint32_t grid, uint32_t species,
                                     double* out, uint64_t n) {
    return guarded([&] {
        need(b, "grid batch");
        need(out, "out");
        alea::grid_download(alea::grid_batch_item(b->impl, grid), species, out, n);
    });
}

alea_status alea_widom_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_ewald* ewald,
                                    const alea_particles* frameworks, const alea_lattice* lattices,
                                    const alea_molecule_species* guests, double temperature,
                                    int32_t precision, alea_widom_batch** out) {
    return guarded([&] {
        need(out, "out");
        *out = nullptr;
        alea::require(lj && frameworks && lattices && guests, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_widom_batch_create: lj, frameworks, lattices and guests are required");
        auto* impl = alea::widom_batch_create(n, lj, ewald, frameworks, lattices, guests, temperature,
                                              precision);
        *out = new alea_widom_batch{impl};
    });
}

alea_status alea_widom_batch_run(alea_widom_batch* b, const uint64_t* seeds, const uint64_t* streams,
                                 uint64_t first_trial, uint64_t n_trials, int32_t draw_order,
                                 alea_widom_result* out, void* cuda_stream) {
    return guarded([&] {
        need(b, "widom batch");
        alea::require(seeds && streams && out, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_widom_batch_run: seeds, streams and out are required");
        alea::widom_batch_run(b->impl, seeds, streams, first_trial, n_trials, draw_order, out,
                              (cudaStream_t)cuda_stream);
    });
}

alea_status alea_widom_batch_destroy(alea_widom_batch* b) {
    return guarded([&] {
        if (!b) return;
        alea::widom_batch_destroy(b->impl);
        delete b;
    });
}

alea_status alea_grid_batch_destroy(alea_grid_batch* b) {
    return guarded([&] {
        if (!b) return;
        alea::grid_batch_destroy(b->impl);
        delete b;
    });
}

alea_status alea_gcmc_set_proposal(alea_gcmc* g, const alea_proposal* p) {
    return guarded([&] {
        need(g, "gcmc");
        if (!p) {
            alea::gcmc_set_proposal(g->impl, nullptr);
            return;
        }
        const alea::ProposalTable t = alea::proposal_table(p->impl);
        alea::gcmc_set_proposal(g->impl, &t);
    });
}

alea_status alea_gcmc_set_grid(alea_gcmc* g, const alea_grid* grid) {
    return guarded([&] {
        need(g, "gcmc");
        alea::gcmc_set_grid(g->impl, grid ? grid->impl : nullptr);
    });
}

alea_status alea_gcmc_set_tail_correction(alea_gcmc* g, int32_t on) {
    return guarded([&] {
        need(g, "gcmc");
        alea::gcmc_set_tail_correction(g->impl, on);
    });
}

alea_status alea_gcmc_set_orientation_trials(alea_gcmc* g, int32_t k) {
    return guarded([&] {
        need(g, "gcmc");
        alea::gcmc_set_orientation_trials(g->impl, k);
    });
}

alea_status alea_widom_set_tail_correction(alea_widom* w, int32_t on, double* du_tail) {
    return guarded([&] {
        need(w, "widom");
        alea::widom_set_tail_correction(w->impl, on);
        if (du_tail) *du_tail = alea::widom_tail_change(w->impl);
    });
}

alea_status alea_gcmc_set_precision(alea_gcmc* g, int32_t precision) {
    return guarded([&] {
        need(g, "gcmc");
        alea::gcmc_set_precision(g->impl, precision);
    });
}

alea_status alea_proposal_create(const alea_proposal_config* config, alea_proposal** out) {
    return guarded([&] {
        need(config, "config");
        need(out, "out");
        *out = nullptr;
        auto* impl = alea::proposal_create(*config);
        *out = new alea_proposal{impl};
    });
}

alea_status alea_proposal_param_count(const alea_proposal* p, uint64_t* out) {
    return guarded([&] {
        need(p, "proposal");
        need(out, "out");
        *out = alea::proposal_param_count(p->impl);
    });
}

alea_status alea_proposal_wave_vectors(const alea_proposal* p, int32_t* out, uint64_t cap) {
    return guarded([&] {
        need(p, "proposal");
        const auto& k = alea::proposal_wave_vectors(p->impl);
        alea::require(out && cap >= k.size(), ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_wave_vectors: output too small");
        std::copy(k.begin(), k.end(), out);
    });
}

alea_status alea_proposal_get_params(const alea_proposal* p, float* out, uint64_t n) {
    return guarded([&] {
        need(p, "proposal");
        alea::require(out && n >= alea::proposal_param_count(p->impl), ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_get_params: output too small");
        alea::proposal_get_params(p->impl, out);
    });
}

alea_status alea_proposal_set_params(alea_proposal* p, const float* in, uint64_t n) {
    return guarded([&] {
        need(p, "proposal");
        alea::require(in && n == alea::proposal_param_count(p->impl), ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_set_params: wrong parameter count");
        alea::proposal_set_params(p->impl, in);
    });
}

alea_status alea_proposal_forward(alea_proposal* p, const float* s, uint64_t n, float* out) {
    return guarded([&] {
        need(p, "proposal");
        alea::require((s && out) || n == 0, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_forward: s and out are required");
        alea::proposal_forward_host(p->impl, s, n, out);
    });
}

alea_status alea_proposal_loss_grad(alea_proposal* p, const float* samples, uint64_t n,
                                    double tau, double* loss, float* grad, uint64_t n_grad) {
    return guarded([&] {
        need(p, "proposal");
        alea::require(samples && loss && grad, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_loss_grad: samples, loss and grad are required");
        alea::require(n_grad >= alea::proposal_param_count(p->impl), ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_loss_grad: gradient output too small");
        *loss = alea::proposal_loss_grad_host(p->impl, samples, n, tau, grad);
    });
}

alea_status alea_proposal_train(alea_proposal* p, const float* samples_device, uint64_t n,
                                const alea_proposal_train_config* config, double* final_loss,
                                void* cuda_stream) {
    return guarded([&] {
        need(p, "proposal");
        alea::require(samples_device && config, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_train: samples_device and config are required");
        const double l = alea::proposal_train(p->impl, samples_device, n, *config,
                                              (cudaStream_t)cuda_stream);
        if (final_loss) *final_loss = l;
    });
}

alea_status alea_proposal_tabulate(alea_proposal* p, uint32_t cells, double uniform_share) {
    return guarded([&] {
        need(p, "proposal");
        alea::proposal_tabulate(p->impl, cells, uniform_share);
    });
}

alea_status alea_proposal_log_density(const alea_proposal* p, const double* s, uint64_t n,
                                      double* out) {
    return guarded([&] {
        need(p, "proposal");
        alea::require((s && out) || n == 0, ALEA_ERR_INVALID_ARGUMENT,
                      "alea_proposal_log_density: s and out are required");
        for (uint64_t i = 0; i < n; ++i) out[i] = alea::proposal_log_density_host(p->impl, s + 3 * i);
    });
}

alea_status alea_proposal_destroy(alea_proposal* p) {
    return guarded([&] {
        if (!p) return;
        alea::proposal_destroy(p->impl);
        delete p;
    });
}

alea_status alea_widom_destroy(alea_widom* w) {
    return guarded([&] {
        if (!w) return;
        alea::widom_destroy(w->impl);
        delete w;
    });
}

// ---------------------------------------------------------------- GCMC chains
alea_status alea_gcmc_create(const alea_lennard_jones* lj, const alea_ewald* ewald,
                             const alea_particles* framework, const alea_lattice* lattice,
                             const alea_molecule_species* species, double temperature,
                             const double* fugacity_pa, const uint64_t* seeds,
                             const uint64_t* streams, uint32_t n_chains, double max_translation,
                             double max_rotation, int32_t draw_order, uint32_t max_molecules,
                             alea_gcmc** out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(species, "species");
        need(fugacity_pa, "fugacity_pa");
        need(seeds, "seeds");
        need(streams, "streams");
        need(out, "out");
        *out = nullptr;
        auto* g = new alea_gcmc{nullptr};
        try {
            g->impl = alea::gcmc_create(*lj, ewald, particles_or_empty(framework), *lattice, 1, species,
                                        temperature, fugacity_pa, seeds, streams, n_chains,
                                        max_translation, max_rotation, draw_order, max_molecules);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

alea_status alea_gcmc_create_mixture(const alea_lennard_jones* lj, const alea_ewald* ewald,
                                     const alea_particles* framework, const alea_lattice* lattice,
                                     uint32_t n_species, const alea_molecule_species* species,
                                     double temperature, const double* fugacity_pa,
                                     const uint64_t* seeds, const uint64_t* streams,
                                     uint32_t n_chains, double max_translation,
                                     double max_rotation, int32_t draw_order,
                                     uint32_t max_molecules, alea_gcmc** out) {
    return guarded([&] {
        need(lj, "lj");
        need(lattice, "lattice");
        need(species, "species");
        need(fugacity_pa, "fugacity_pa");
        need(seeds, "seeds");
        need(streams, "streams");
        need(out, "out");
        *out = nullptr;
        auto* g = new alea_gcmc{nullptr};
        try {
            g->impl = alea::gcmc_create(*lj, ewald, particles_or_empty(framework), *lattice, n_species,
                                        species, temperature, fugacity_pa, seeds, streams, n_chains,
                                        max_translation, max_rotation, draw_order, max_molecules);
        } catch (...) {
            delete g;
            throw;
        }
        *out = g;
    });
}

alea_status alea_gcmc_run(alea_gcmc* g, uint64_t steps, void* cuda_stream) {
    return guarded([&] {
        need(g, "gcmc");
        alea::gcmc_run(g->impl, steps, (cudaStream_t)cuda_stream);
    });
}

alea_status alea_gcmc_chain_info_get(const alea_gcmc* g, uint32_t chain, alea_gcmc_chain_info* out) {
    return guarded([&] {
        need(g, "gcmc");
        need(out, "out");
        const unsigned n = alea::gcmc_chains(g->impl);
        if (chain >= n) throw alea::Error(ALEA_ERR_OUT_OF_RANGE, "GCMC: chain index");
        std::vector<alea::ChainState> st(n);
        alea::gcmc_states(g->impl, st.data());
        const alea::ChainState& c = st[chain];
        out->molecules = c.n_mol;
        out->guest_sites = c.n_guest;
        out->call_index = c.call;
        out->steps = c.steps;
        out->resyncs = c.resyncs;
        for (int i = 0; i < 5; ++i) {
            out->attempted[i] = c.attempted[i];
            out->accepted[i] = c.accepted[i];
        }
        for (int i = 0; i < 4; ++i) out->species_molecules[i] = c.n_of[i];
        out->sum_molecules = c.sum_n;
        out->sum_molecules_sq = c.sum_n2;
        out->last_du = c.last_du;
        out->last_kernel_ms = alea::gcmc_last_ms(g->impl);
    });
}

alea_status alea_gcmc_particles(const alea_gcmc* g, uint32_t chain, double* xyz, uint64_t cap,
                                uint64_t* n_out) {
    return guarded([&] {
        need(g, "gcmc");
        const uint64_t n = alea::gcmc_particles(g->impl, chain, xyz, cap);
        if (n_out) *n_out = n;
    });
}

alea_status alea_gcmc_guest_sites(const alea_gcmc* g, uint32_t chain, double* xyzq,
                                  uint32_t* lj_species, uint64_t cap, uint64_t* n_out) {
    return guarded([&] {
        need(g, "gcmc");
        const uint64_t n = alea::gcmc_guest_sites(g->impl, chain, xyzq, lj_species, cap);
        if (n_out) *n_out = n;
    });
}

alea_status alea_gcmc_ewald_energy(const alea_gcmc* g, uint32_t chain, double* out) {
    return guarded([&] {
        need(g, "gcmc");
        need(out, "out");
        *out = alea::gcmc_ewald_energy(g->impl, chain);
    });
}

alea_status alea_gcmc_destroy(alea_gcmc* g) {
    return guarded([&] {
        if (!g) return;
        alea::gcmc_destroy(g->impl);
        delete g;
    });
}

// ---------------------------------------------------------------- acceptance / EOS
double alea_insertion_ratio(double f, double v, uint64_t n_before, double t, double du) {
    return (f * v / t) / (double)(n_before + 1) * std::exp(-du / t);
}
double alea_deletion_ratio(double f, double v, uint64_t n_before, double t, double du) {
    return (double)n_before / (f * v / t) * std::exp(-du / t);
}
double alea_metropolis_ratio(double t, double du) { return std::exp(-du / t); }
double alea_swap_ratio(double f_from, double f_to, uint64_t n_from, uint64_t n_to, double t,
                       double du) {
    return (f_to / f_from) * ((double)n_from / (double)(n_to + 1)) * std::exp(-du / t);
}

// The gas-phase root of Z^3 - (1-B) Z^2 + (A - 3B^2 - 2B) Z - (AB - B^2 - B^3):
// Newton from Z = 1, kept above B (peng_robinson.cc:62-100; the mixture's
// solve, :236-276, is the same with the mixture's A and B).
static double pr_gas_root(double A, double B, const char* who, double t, double p) {
    const double c2 = -(1.0 - B), c1 = A - 3.0 * B * B - 2.0 * B, c0 = -(A * B - B * B - B * B * B);
    double z = 1.0;
    bool converged = false;
    for (int it = 0; it < 100; ++it) {
        const double fz = z * z * z + c2 * z * z + c1 * z + c0;
        if (std::fabs(fz) < 1e-14) {
            converged = true;
            break;
        }
        const double fp = 3.0 * z * z + 2.0 * c2 * z + c1;
        if (fp == 0.0) break;
        z -= fz / fp;
        if (!(z > B)) z = B + 0.5 * (1.0 - B > 0 ? 1.0 - B : 1.0);
    }
    if (!converged && std::fabs(z * z * z + c2 * z * z + c1 * z + c0) > 1e-8)
        throw alea::Error(ALEA_ERR_RUNTIME, std::string(who) + ": Newton-Raphson did not converge for T=" +
                                                std::to_string(t) + " K, P=" + std::to_string(p) + " Pa");
    return z;
}

// PengRobinson (peng_robinson.cc:10-110): a scalar Newton solve, host side.
alea_status alea_peng_robinson_fugacity(double tc, double pc, double omega, double t, double p,
                                        double* out) {
    return guarded([&] {
        need(out, "out");
        if (!(tc > 0.0)) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "PengRobinson: criticalTemperatureKelvin must be positive");
        if (!(pc > 0.0)) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "PengRobinson: criticalPressurePascal must be positive");
        if (!(t > 0.0)) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "PengRobinson: temperatureKelvin must be positive");
        if (!(p > 0.0)) throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, "PengRobinson: pressurePascal must be positive");
        const double R = 8.31446261815324;
        const double a = 0.45724 * R * R * tc * tc / pc;
        const double b = 0.07780 * R * tc / pc;
        const double kappa = 0.37464 + 1.54226 * omega - 0.26992 * omega * omega;
        const double term = 1.0 + kappa * (1.0 - std::sqrt(t / tc));
        const double aa = a * (term * term);
        const double A = aa * p / (R * R * t * t);
        const double B = b * p / (R * t);
        const double z = pr_gas_root(A, B, "PengRobinson::compressibilityFactor", t, p);
        const double s2 = 1.41421356237309504880;
        const double lnphi = (z - 1.0) - std::log(z - B) -
                             (A / (2.0 * s2 * B)) * std::log((z + (1.0 + s2) * B) / (z + (1.0 - s2) * B));
        *out = std::exp(lnphi) * p;
    });
}

// PengRobinsonMixture (peng_robinson.cc:112-309): van der Waals one-fluid
// mixing, a_ij = sqrt(a_i(T) a_j(T)) (1 - k_ij), a_mix = sum x_i x_j a_ij,
// b_mix = sum x_i b_i; the mixture's Z from the pure form's cubic; per
// component f_i = x_i phi_i P with ln phi_i = (b_i/b)(Z-1) - ln(Z-B)
// - A/(2 sqrt2 B) [(2/a) sum_j x_j a_ij - b_i/b] ln[(Z+(1+sqrt2)B)/(Z+(1-sqrt2)B)].
alea_status alea_peng_robinson_mixture(uint32_t n, const double* tc, const double* pc,
                                       const double* omega, const double* kij, double t, double p,
                                       const double* x, double* z_out, double* f_out) {
    return guarded([&] {
        auto bad = [](const std::string& m) { throw alea::Error(ALEA_ERR_INVALID_ARGUMENT, m); };
        if (n < 2) bad("PengRobinsonMixture: needs at least 2 substances (use PengRobinson for a pure component)");
        need(tc, "tc");
        need(pc, "pc");
        need(omega, "omega");
        need(x, "mole_fractions");
        need(f_out, "out");
        const double R = 8.31446261815324;
        std::vector<double> a(n), b(n), kappa(n);
        for (uint32_t i = 0; i < n; ++i) {
            if (!(tc[i] > 0.0)) bad("PengRobinsonMixture: criticalTemperatureKelvin must be positive");
            if (!(pc[i] > 0.0)) bad("PengRobinsonMixture: criticalPressurePascal must be positive");
            a[i] = 0.45724 * R * R * tc[i] * tc[i] / pc[i];
            b[i] = 0.07780 * R * tc[i] / pc[i];
            kappa[i] = 0.37464 + 1.54226 * omega[i] - 0.26992 * omega[i] * omega[i];
        }
        // k_ij: n x n, zero diagonal, symmetric (NULL: every k_ij = 0)
        auto k = [&](uint32_t i, uint32_t j) { return kij ? kij[(size_t)i * n + j] : 0.0; };
        if (kij)
            for (uint32_t i = 0; i < n; ++i) {
                if (kij[(size_t)i * n + i] != 0.0)
                    bad("PengRobinsonMixture: binaryInteractionKij diagonal must be zero (k_ii = 0)");
                for (uint32_t j = i + 1; j < n; ++j)
                    if (kij[(size_t)i * n + j] != kij[(size_t)j * n + i])
                        bad("PengRobinsonMixture: binaryInteractionKij must be symmetric (k_ij = k_ji)");
            }
        // fugacitiesPascal checks the mole fractions, then compressibilityFactor T and P
        double sum = 0.0;
        for (uint32_t i = 0; i < n; ++i) {
            if (!(x[i] >= 0.0)) bad("PengRobinsonMixture: every mole fraction must be >= 0");
            sum += x[i];
        }
        if (std::fabs(sum - 1.0) > 1e-9)
            bad("PengRobinsonMixture: mole fractions must sum to 1 (got " + std::to_string(sum) + ")");
        if (!(t > 0.0)) bad("PengRobinsonMixture: temperatureKelvin must be positive");
        if (!(p > 0.0)) bad("PengRobinsonMixture: totalPressurePascal must be positive");
        std::vector<double> aa(n);
        for (uint32_t i = 0; i < n; ++i) {
            const double term = 1.0 + kappa[i] * (1.0 - std::sqrt(t / tc[i]));
            aa[i] = a[i] * (term * term);
        }
        // a_mix as compressibilityFactor forms it (x_i x_j a_ij) and as
        // fugacitiesPascal does ((x_i x_j sqrt(..)) (1 - k_ij)); their last bits can differ
        double amix_z = 0.0, amix = 0.0, bmix = 0.0;
        for (uint32_t i = 0; i < n; ++i) {
            bmix += x[i] * b[i];
            for (uint32_t j = 0; j < n; ++j) {
                const double g = std::sqrt(aa[i] * aa[j]);
                amix_z += x[i] * x[j] * (g * (1.0 - k(i, j)));
                amix += x[i] * x[j] * g * (1.0 - k(i, j));
            }
        }
        const double Az = amix_z * p / (R * R * t * t);
        const double B = bmix * p / (R * t);
        const double z = pr_gas_root(Az, B, "PengRobinsonMixture::compressibilityFactor", t, p);
        const double A = amix * p / (R * R * t * t);
        const double s2 = 1.41421356237309504880;
        for (uint32_t i = 0; i < n; ++i) {
            double sj = 0.0;
            for (uint32_t j = 0; j < n; ++j) sj += x[j] * std::sqrt(aa[i] * aa[j]) * (1.0 - k(i, j));
            const double lnphi = (b[i] / bmix) * (z - 1.0) - std::log(z - B) -
                                 (A / (2.0 * s2 * B)) * ((2.0 / amix) * sj - b[i] / bmix) *
                                     std::log((z + (1.0 + s2) * B) / (z + (1.0 - s2) * B));
            f_out[i] = x[i] * std::exp(lnphi) * p;
        }
        if (z_out) *z_out = z;
    });
}

}  // extern "C"

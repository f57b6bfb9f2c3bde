// Test infrastructure only: a plain C-ABI shim over the reference engine's own
// classes, compiled together with the reference's hot-path translation units
// (straight from their sources, see oracle/build_ref.sh) into
// oracle/_ref/libaleator_ref.so. The parity tests and the golden-vector script
// use it to pin the C restatement (oracle/aleator_oracle.c) and the CUDA path
// against the reference itself. It is never linked into the product.
//
// Every function here calls the reference's public API; the only logic of its
// own is argument marshalling and, for per-trial Widom energies, a replay of
// monte_carlo_engine.cc:881-910 built from the same public calls (checked
// bit-for-bit against MonteCarloEngine::widomInsertionHenryCoefficient).

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <memory>
#include <numbers>
#include <vector>

#include "core/geometry/lattice.hpp"
#include "core/geometry/supercell.hpp"
#include "core/math/counter_based_rng.hpp"
#include "core/math/particle_data.hpp"
#include "core/neighbor/verlet_list.hpp"
#include "engines/monte_carlo/framework_energy_grid.hpp"
#include "engines/monte_carlo/molecule_species.hpp"
#include "engines/monte_carlo/monte_carlo_engine.hpp"
#include "engines/monte_carlo/peng_robinson.hpp"
#include "forcefield/electrostatics/ewald.hpp"
#include "forcefield/electrostatics/ewald_incremental_state.hpp"
#include "forcefield/pairwise/lennard_jones.hpp"
#include "io/structure_io.hpp"

using namespace aleator;

namespace {

core::Lattice latticeOf(const double* m) {
    std::array<std::array<double, 3>, 3> a{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = m[3 * i + j];
    return core::Lattice(a);
}

core::ParticleData particlesOf(uint64_t n, const double* x, const double* y, const double* z,
                               const double* q, const uint32_t* sp) {
    core::ParticleData p;
    for (uint64_t i = 0; i < n; ++i)
        p.push_back(x[i], y[i], z[i], 0.0, 0.0, 0.0, 1.0, q ? q[i] : 0.0, sp ? sp[i] : 0u);
    return p;
}

std::shared_ptr<forcefield::LennardJones> ljOf(uint32_t nSpecies, const double* eps,
                                               const double* sigma, double cutoff, int trunc,
                                               int mixing) {
    std::vector<forcefield::LennardJonesParameters> params(nSpecies);
    for (uint32_t i = 0; i < nSpecies; ++i) params[i] = {eps[i], sigma[i]};
    return std::make_shared<forcefield::LennardJones>(
        params, cutoff, static_cast<forcefield::LennardJonesTruncation>(trunc),
        static_cast<forcefield::MixingRule>(mixing));
}

std::vector<forcefield::ChargedSite> sitesOf(const double* s, uint64_t n) {
    std::vector<forcefield::ChargedSite> v(n);
    for (uint64_t i = 0; i < n; ++i) v[i] = {s[4 * i], s[4 * i + 1], s[4 * i + 2], s[4 * i + 3]};
    return v;
}

engines::MoleculeSpecies speciesOf(uint32_t nSites, const double* sx, const double* sy,
                                   const double* sz, const uint32_t* lj, const double* q) {
    engines::MoleculeSpecies sp;
    for (uint32_t i = 0; i < nSites; ++i) sp.sites.push_back({sx[i], sy[i], sz[i], lj[i], q[i], 1.0});
    return sp;
}

std::vector<std::vector<std::size_t>> moleculesOf(uint64_t nMol, const uint64_t* offsets,
                                                  const uint64_t* indices) {
    std::vector<std::vector<std::size_t>> m(nMol);
    for (uint64_t k = 0; k < nMol; ++k)
        for (uint64_t j = offsets[k]; j < offsets[k + 1]; ++j) m[k].push_back(indices[j]);
    return m;
}

using Vec3 = std::array<double, 3>;

}  // namespace

extern "C" {

// ---------------------------------------------------------------- Philox
void ref_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    const auto r = core::philox4x32_10({ctr[0], ctr[1], ctr[2], ctr[3]}, {key[0], key[1]});
    for (int i = 0; i < 4; ++i) out[i] = r[i];
}

void ref_philox_u64(uint64_t seed, uint64_t stream, uint64_t skip, uint64_t n, uint64_t* out) {
    core::Philox4x32Rng rng;
    rng.seed(seed, stream);
    for (uint64_t i = 0; i < skip; ++i) (void)rng.nextU64();
    for (uint64_t i = 0; i < n; ++i) out[i] = rng.nextU64();
}

void ref_philox_uniform(uint64_t seed, uint64_t stream, uint64_t skip, uint64_t n, double* out) {
    core::Philox4x32Rng rng;
    rng.seed(seed, stream);
    for (uint64_t i = 0; i < skip; ++i) (void)rng.nextU64();
    for (uint64_t i = 0; i < n; ++i) out[i] = rng.nextUniform();
}

// ---------------------------------------------------------------- Lattice
void ref_min_image(const double* m, const double* a, const double* b, uint64_t n, double* out) {
    const auto lat = latticeOf(m);
    for (uint64_t i = 0; i < n; ++i) {
        const auto d = lat.minimumImageDisplacement({a[3 * i], a[3 * i + 1], a[3 * i + 2]},
                                                    {b[3 * i], b[3 * i + 1], b[3 * i + 2]});
        out[3 * i] = d[0];
        out[3 * i + 1] = d[1];
        out[3 * i + 2] = d[2];
    }
}

double ref_perpendicular_width(const double* m, int axis) {
    return latticeOf(m).perpendicularWidth(axis);
}

void ref_supercell_replication(const double* m, double cutoff, int* out) {
    const auto n = core::minimumSupercellReplication(latticeOf(m), cutoff);
    out[0] = n[0];
    out[1] = n[1];
    out[2] = n[2];
}

// ---------------------------------------------------------------- Lennard-Jones
double ref_lj_pair_energy(double r, double eps, double sigma, double cutoff, int trunc) {
    const double e[1] = {eps};
    const double s[1] = {sigma};
    return ljOf(1, e, s, cutoff, trunc, 0)->pairEnergy(r, {eps, sigma});
}

void ref_lj_mixed(uint32_t nSpecies, const double* eps, const double* sigma, int mixing,
                  uint32_t i, uint32_t j, double* out) {
    const auto p = ljOf(nSpecies, eps, sigma, 1.0, 0, mixing)->mixedParameters(i, j);
    out[0] = p.epsilon;
    out[1] = p.sigma;
}

// Per-particle LJ energy (LennardJones::computeParticleEnergy) for each
// query index, excluding `excluded`.
void ref_lj_particle_energy(const double* m, uint64_t n, const double* x, const double* y,
                            const double* z, const uint32_t* sp, uint32_t nSpecies,
                            const double* eps, const double* sigma, double cutoff, int trunc,
                            int mixing, const uint64_t* query, uint64_t nQuery,
                            const uint64_t* excluded, uint64_t nExcluded, double* out) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, nullptr, sp);
    const auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::vector<std::size_t> ex(excluded, excluded + nExcluded);
    for (uint64_t k = 0; k < nQuery; ++k) out[k] = lj->computeParticleEnergy(query[k], p, lat, ex);
}

void ref_lj_energy_virial(const double* m, uint64_t n, const double* x, const double* y,
                          const double* z, double eps, double sigma, double cutoff, int trunc,
                          double* out) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, nullptr, nullptr);
    const double e[1] = {eps};
    const double s[1] = {sigma};
    const auto lj = ljOf(1, e, s, cutoff, trunc, 0);
    core::VerletList nl(0.5);
    nl.build(p, lat, cutoff);
    out[0] = lj->computeEnergy(p, lat, nl);
    out[1] = lj->computeVirial(p, lat, nl);
    out[2] = lj->tailEnergyCorrection(p, lat);
}

double ref_lj_tail(const double* m, uint64_t n, const uint32_t* sp, uint32_t nSpecies,
                   const double* eps, const double* sigma, double cutoff, int mixing) {
    const auto lat = latticeOf(m);
    std::vector<double> zeros(n, 0.0);
    const auto p = particlesOf(n, zeros.data(), zeros.data(), zeros.data(), nullptr, sp);
    return ljOf(nSpecies, eps, sigma, cutoff, 0, mixing)->tailEnergyCorrection(p, lat);
}

// ---------------------------------------------------------------- Energy grid
void* ref_grid_create(const double* m, uint64_t n, const double* x, const double* y,
                      const double* z, const uint32_t* sp, uint32_t nSpecies, const double* eps,
                      const double* sigma, double cutoff, int trunc, int mixing,
                      const uint32_t* guest, uint32_t nGuest, double spacing) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, nullptr, sp);
    const auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::vector<uint32_t> g(guest, guest + nGuest);
    return new engines::FrameworkEnergyGrid(*lj, p, lat, g, spacing);
}

void ref_grid_counts(void* h, int* out) {
    const auto c = static_cast<engines::FrameworkEnergyGrid*>(h)->pointCounts();
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
}

void ref_grid_interpolate(void* h, uint32_t species, const double* xyz, uint64_t n, double* out) {
    const auto* g = static_cast<engines::FrameworkEnergyGrid*>(h);
    for (uint64_t i = 0; i < n; ++i)
        out[i] = g->interpolate(species, {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
}

// Writes the reference's own cache file for this grid (the key is rebuilt
// from the same inputs, exactly as loadOrBuildFrameworkEnergyGrid does).
int ref_grid_serialize(void* h, const char* path, const double* m, uint64_t n, const double* x,
                       const double* y, const double* z, const uint32_t* sp, uint32_t nSpecies,
                       const double* eps, const double* sigma, double cutoff, int trunc,
                       int mixing, const uint32_t* guest, uint32_t nGuest, double spacing) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, nullptr, sp);
    const auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::vector<uint32_t> g(guest, guest + nGuest);
    const auto key = engines::makeFrameworkEnergyGridCacheKey(*lj, p, lat, g, spacing);
    static_cast<engines::FrameworkEnergyGrid*>(h)->serialize(path, key);
    return 0;
}

// Content-addressed cache file name for the same key (cacheFilePath).
int ref_grid_cache_name(char* out, uint64_t cap, const double* m, uint64_t n, const double* x,
                        const double* y, const double* z, const uint32_t* sp, uint32_t nSpecies,
                        const double* eps, const double* sigma, double cutoff, int trunc,
                        int mixing, const uint32_t* guest, uint32_t nGuest, double spacing) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, nullptr, sp);
    const auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::vector<uint32_t> g(guest, guest + nGuest);
    const auto key = engines::makeFrameworkEnergyGridCacheKey(*lj, p, lat, g, spacing);
    const std::string name = engines::FrameworkEnergyGrid::cacheFilePath("", key).string();
    std::snprintf(out, cap, "%s", name.c_str());
    return 0;
}

void ref_grid_destroy(void* h) { delete static_cast<engines::FrameworkEnergyGrid*>(h); }

// ---------------------------------------------------------------- Ewald
uint64_t ref_ewald_terms(const double* m, double alpha, int kMax, double* k, double* w,
                         uint64_t cap) {
    const forcefield::Ewald ewald(alpha, 1.0, kMax);
    const auto terms = ewald.reciprocalTerms(latticeOf(m));
    for (uint64_t t = 0; t < terms.size() && t < cap; ++t) {
        k[3 * t] = terms[t].k[0];
        k[3 * t + 1] = terms[t].k[1];
        k[3 * t + 2] = terms[t].k[2];
        w[t] = terms[t].weight;
    }
    return terms.size();
}

// Ewald::computeEnergyBreakdown -> out = {real, reciprocal, self, exclusion, surface}.
void ref_ewald_breakdown(const double* m, uint64_t n, const double* x, const double* y,
                         const double* z, const double* q, double alpha, double rc, int kMax,
                         const uint64_t* exclusions, uint64_t nExcl, double skin, double* out) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, q, nullptr);
    std::vector<std::pair<std::size_t, std::size_t>> ex;
    for (uint64_t i = 0; i < nExcl; ++i) ex.emplace_back(exclusions[2 * i], exclusions[2 * i + 1]);
    const forcefield::Ewald ewald(alpha, rc, kMax, ex);
    core::VerletList nl(skin);
    nl.build(p, lat, rc);
    const auto b = ewald.computeEnergyBreakdown(p, lat, nl);
    out[0] = b.real;
    out[1] = b.reciprocal;
    out[2] = b.self;
    out[3] = b.exclusion;
    out[4] = b.surface;
}

void ref_ewald_real_space_particle_energy(const double* m, uint64_t n, const double* x,
                                          const double* y, const double* z, const double* q,
                                          double alpha, double rc, const uint64_t* query,
                                          uint64_t nQuery, const uint64_t* excluded,
                                          uint64_t nExcluded, double* out) {
    const auto lat = latticeOf(m);
    const auto p = particlesOf(n, x, y, z, q, nullptr);
    const forcefield::Ewald ewald(alpha, rc, 1);
    std::vector<std::size_t> ex(excluded, excluded + nExcluded);
    for (uint64_t k = 0; k < nQuery; ++k)
        out[k] = ewald.realSpaceParticleEnergy(query[k], p, lat, ex);
}

struct RefEwaldState {
    core::Lattice lattice;
    forcefield::Ewald ewald;
    std::unique_ptr<forcefield::EwaldIncrementalState> state;
};

void* ref_ews_create(const double* m, uint64_t n, const double* x, const double* y,
                     const double* z, const double* q, double alpha, double rc, int kMax) {
    auto* s = new RefEwaldState{latticeOf(m), forcefield::Ewald(alpha, rc, kMax), nullptr};
    const auto p = particlesOf(n, x, y, z, q, nullptr);
    s->state = std::make_unique<forcefield::EwaldIncrementalState>(s->ewald, p, s->lattice);
    return s;
}

double ref_ews_energy(void* h) { return static_cast<RefEwaldState*>(h)->state->committedEnergy(); }

double ref_ews_propose(void* h, const double* removed, uint64_t nr, const double* added,
                       uint64_t na) {
    auto* s = static_cast<RefEwaldState*>(h);
    const auto r = sitesOf(removed, nr);
    const auto a = sitesOf(added, na);
    if (nr == 0) return s->state->proposeInsertion(a);
    if (na == 0) return s->state->proposeDeletion(r);
    return s->state->proposeMove(r, a);
}

void ref_ews_commit(void* h, const double* removed, uint64_t nr, const double* added,
                    uint64_t na) {
    auto* s = static_cast<RefEwaldState*>(h);
    const auto r = sitesOf(removed, nr);
    const auto a = sitesOf(added, na);
    if (nr == 0)
        s->state->commitInsertion(a);
    else if (na == 0)
        s->state->commitDeletion(r);
    else
        s->state->commitMove(r, a);
}

double ref_ews_recompute(void* h, uint64_t n, const double* x, const double* y, const double* z,
                         const double* q, uint64_t nMol, const uint64_t* offsets,
                         const uint64_t* indices) {
    auto* s = static_cast<RefEwaldState*>(h);
    const auto p = particlesOf(n, x, y, z, q, nullptr);
    return s->state->recomputeFromScratch(p, moleculesOf(nMol, offsets, indices));
}

void ref_ews_resync(void* h, uint64_t n, const double* x, const double* y, const double* z,
                    const double* q, uint64_t nMol, const uint64_t* offsets,
                    const uint64_t* indices) {
    auto* s = static_cast<RefEwaldState*>(h);
    const auto p = particlesOf(n, x, y, z, q, nullptr);
    s->state->resync(p, moleculesOf(nMol, offsets, indices));
}

uint64_t ref_ews_raw(void* h, double* out, uint64_t cap) {
    const auto raw = static_cast<RefEwaldState*>(h)->state->rawStateForTesting();
    for (uint64_t i = 0; i < raw.size() && i < cap; ++i) out[i] = raw[i];
    return raw.size();
}

void ref_ews_destroy(void* h) { delete static_cast<RefEwaldState*>(h); }

// ---------------------------------------------------------------- Widom / GCMC
struct RefSystem {
    core::ParticleData framework;
    core::Lattice lattice;
    std::shared_ptr<forcefield::LennardJones> lj;
    std::shared_ptr<forcefield::Ewald> ewald;
    engines::MoleculeSpecies species;
};

// Henry coefficient through MonteCarloEngine::widomInsertionHenryCoefficient
// (the public API), and, when perTrial != nullptr, each trial's deltaU from a
// replay of monte_carlo_engine.cc:881-910 using the same public calls on a
// second RNG with the same (seed, stream). Returns {engine K_H, replay K_H}.
void ref_widom(const double* m, uint64_t n, const double* x, const double* y, const double* z,
               const double* q, const uint32_t* sp, uint32_t nSpecies, const double* eps,
               const double* sigma, double cutoff, int trunc, int mixing, double alpha,
               double ewaldRc, int kMax, uint32_t nSites, const double* sx, const double* sy,
               const double* sz, const uint32_t* sLj, const double* sq, double temperature,
               uint64_t seed, uint64_t stream, uint64_t nTrials, double* perTrial,
               double* khOut, int reversedDraws) {
    const auto lat = latticeOf(m);
    const auto fw = particlesOf(n, x, y, z, q, sp);
    auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::shared_ptr<forcefield::Ewald> ewald;
    if (alpha > 0.0) ewald = std::make_shared<forcefield::Ewald>(alpha, ewaldRc, kMax);
    const auto species = speciesOf(nSites, sx, sy, sz, sLj, sq);

    auto rng = std::make_unique<core::Philox4x32Rng>();
    rng->seed(seed, stream);
    engines::MonteCarloEngine engine(fw, lat, lj, std::move(rng), temperature, species, 1.0, 1.5,
                                     0.5, ewald, nullptr);
    khOut[0] = engine.widomInsertionHenryCoefficient(nTrials);
    if (perTrial == nullptr) {
        khOut[1] = khOut[0];
        return;
    }

    // Replay with the same primitives, recording each trial's deltaU.
    core::Philox4x32Rng r;
    r.seed(seed, stream);
    core::ParticleData work = fw;
    std::unique_ptr<forcefield::EwaldIncrementalState> ews;
    if (ewald) ews = std::make_unique<forcefield::EwaldIncrementalState>(*ewald, work, lat);
    const auto& mat = lat.matrix();
    double sum = 0.0;
    for (uint64_t t = 0; t < nTrials; ++t) {
        double u0 = r.nextUniform();
        double u1 = r.nextUniform();
        double u2 = r.nextUniform();
        if (reversedDraws) std::swap(u0, u2);
        Vec3 ref{};
        for (int c = 0; c < 3; ++c) ref[c] = (mat[0][c] * u0 + mat[1][c] * u1) + mat[2][c] * u2;
        double qw = 1.0, qx = 0.0, qy = 0.0, qz = 0.0;
        if (nSites > 1) {
            double v0 = r.nextUniform();
            double v1 = r.nextUniform();
            double v2 = r.nextUniform();
            if (reversedDraws) std::swap(v0, v2);
            const double r1 = std::sqrt(1.0 - v0);
            const double r2 = std::sqrt(v0);
            const double t1 = 2.0 * std::numbers::pi * v1;
            const double t2 = 2.0 * std::numbers::pi * v2;
            qw = r2 * std::cos(t2);
            qx = r1 * std::sin(t1);
            qy = r1 * std::cos(t1);
            qz = r2 * std::sin(t2);
        }
        std::vector<std::size_t> idx;
        for (uint32_t s = 0; s < nSites; ++s) {
            Vec3 v{sx[s], sy[s], sz[s]};
            if (nSites > 1) {
                const Vec3 tt{2.0 * (qy * v[2] - qz * v[1]), 2.0 * (qz * v[0] - qx * v[2]),
                              2.0 * (qx * v[1] - qy * v[0])};
                const Vec3 c2{qy * tt[2] - qz * tt[1], qz * tt[0] - qx * tt[2],
                              qx * tt[1] - qy * tt[0]};
                v = {(v[0] + tt[0] * qw) + c2[0], (v[1] + tt[1] * qw) + c2[1],
                     (v[2] + tt[2] * qw) + c2[2]};
            }
            idx.push_back(work.push_back(ref[0] + v[0], ref[1] + v[1], ref[2] + v[2], 0.0, 0.0,
                                         0.0, 1.0, sq[s], sLj[s]));
        }
        double dU = 0.0;
        for (std::size_t s : idx) dU += lj->computeParticleEnergy(s, work, lat, idx);
        if (ewald) {
            double e = 0.0;
            for (std::size_t s : idx) e += ewald->realSpaceParticleEnergy(s, work, lat, idx);
            dU += e;
            std::vector<forcefield::ChargedSite> cs;
            for (std::size_t s : idx) cs.push_back({work.x[s], work.y[s], work.z[s], work.charge[s]});
            dU += ews->proposeInsertion(cs);
        }
        perTrial[t] = dU;
        sum += std::exp(-dU / temperature);
        for (uint32_t s = 0; s < nSites; ++s) work.popBack();
    }
    khOut[1] = (sum / static_cast<double>(nTrials)) / temperature;
}

struct RefGcmc {
    core::Lattice lattice;
    std::unique_ptr<engines::MonteCarloEngine> engine;
};

void* ref_gcmc_create(const double* m, uint64_t n, const double* x, const double* y,
                      const double* z, const double* q, const uint32_t* sp, uint32_t nSpecies,
                      const double* eps, const double* sigma, double cutoff, int trunc,
                      int mixing, double alpha, double ewaldRc, int kMax, uint32_t nSites,
                      const double* sx, const double* sy, const double* sz, const uint32_t* sLj,
                      const double* sq, double temperature, double fugacityPa, double maxTrans,
                      double maxRot, uint64_t seed, uint64_t stream) {
    auto* g = new RefGcmc{latticeOf(m), nullptr};
    const auto fw = particlesOf(n, x, y, z, q, sp);
    auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::shared_ptr<forcefield::Ewald> ewald;
    if (alpha > 0.0) ewald = std::make_shared<forcefield::Ewald>(alpha, ewaldRc, kMax);
    auto rng = std::make_unique<core::Philox4x32Rng>();
    rng->seed(seed, stream);
    g->engine = std::make_unique<engines::MonteCarloEngine>(
        fw, g->lattice, lj, std::move(rng), temperature, speciesOf(nSites, sx, sy, sz, sLj, sq),
        fugacityPa, maxTrans, maxRot, ewald, nullptr);
    return g;
}

// The same chain with the engine's shared FrameworkEnergyGrid built by the
// reference from the same inputs (monte_carlo_engine.hpp:76-83).
void* ref_gcmc_create_grid(const double* m, uint64_t n, const double* x, const double* y,
                           const double* z, const double* q, const uint32_t* sp, uint32_t nSpecies,
                           const double* eps, const double* sigma, double cutoff, int trunc,
                           int mixing, double alpha, double ewaldRc, int kMax, uint32_t nSites,
                           const double* sx, const double* sy, const double* sz, const uint32_t* sLj,
                           const double* sq, double temperature, double fugacityPa, double maxTrans,
                           double maxRot, uint64_t seed, uint64_t stream, double spacing,
                           uint32_t nGrid, const uint32_t* gridSpecies) {
    auto* g = new RefGcmc{latticeOf(m), nullptr};
    const auto fw = particlesOf(n, x, y, z, q, sp);
    auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::shared_ptr<forcefield::Ewald> ewald;
    if (alpha > 0.0) ewald = std::make_shared<forcefield::Ewald>(alpha, ewaldRc, kMax);
    const std::vector<uint32_t> ids(gridSpecies, gridSpecies + nGrid);
    auto grid = std::make_shared<const engines::FrameworkEnergyGrid>(*lj, fw, g->lattice, ids, spacing);
    auto rng = std::make_unique<core::Philox4x32Rng>();
    rng->seed(seed, stream);
    g->engine = std::make_unique<engines::MonteCarloEngine>(
        fw, g->lattice, lj, std::move(rng), temperature, speciesOf(nSites, sx, sy, sz, sLj, sq),
        fugacityPa, maxTrans, maxRot, ewald, grid);
    return g;
}

// The mixture constructor (monte_carlo_engine.hpp:143-151): nGuest species,
// species k with nSitesPer[k] sites, their site arrays concatenated; with
// nGrid > 0, the engine's FrameworkEnergyGrid of those species at `spacing`.
void* ref_gcmc_create_mixture(const double* m, uint64_t n, const double* x, const double* y,
                              const double* z, const double* q, const uint32_t* sp,
                              uint32_t nSpecies, const double* eps, const double* sigma,
                              double cutoff, int trunc, int mixing, double alpha, double ewaldRc,
                              int kMax, uint32_t nGuest, const uint32_t* nSitesPer,
                              const double* sx, const double* sy, const double* sz,
                              const uint32_t* sLj, const double* sq, const double* fugacitiesPa,
                              double temperature, double maxTrans, double maxRot, uint64_t seed,
                              uint64_t stream, double spacing, uint32_t nGrid,
                              const uint32_t* gridSpecies) {
    auto* g = new RefGcmc{latticeOf(m), nullptr};
    const auto fw = particlesOf(n, x, y, z, q, sp);
    auto lj = ljOf(nSpecies, eps, sigma, cutoff, trunc, mixing);
    std::shared_ptr<forcefield::Ewald> ewald;
    if (alpha > 0.0) ewald = std::make_shared<forcefield::Ewald>(alpha, ewaldRc, kMax);
    std::vector<engines::MoleculeSpecies> list;
    std::vector<double> fug;
    uint32_t off = 0;
    for (uint32_t k = 0; k < nGuest; ++k) {
        list.push_back(speciesOf(nSitesPer[k], sx + off, sy + off, sz + off, sLj + off, sq + off));
        fug.push_back(fugacitiesPa[k]);
        off += nSitesPer[k];
    }
    std::shared_ptr<const engines::FrameworkEnergyGrid> grid;
    if (nGrid > 0) {
        const std::vector<uint32_t> ids(gridSpecies, gridSpecies + nGrid);
        grid = std::make_shared<const engines::FrameworkEnergyGrid>(*lj, fw, g->lattice, ids, spacing);
    }
    auto rng = std::make_unique<core::Philox4x32Rng>();
    rng->seed(seed, stream);
    g->engine = std::make_unique<engines::MonteCarloEngine>(fw, g->lattice, lj, std::move(rng),
                                                            temperature, list, fug, maxTrans,
                                                            maxRot, ewald, grid);
    return g;
}

uint64_t ref_gcmc_molecules_of(void* h, uint64_t species) {
    return static_cast<RefGcmc*>(h)->engine->moleculeCountOfSpecies(species);
}

void ref_gcmc_run(void* h, uint64_t steps) { static_cast<RefGcmc*>(h)->engine->run(steps); }

uint64_t ref_gcmc_molecules(void* h) { return static_cast<RefGcmc*>(h)->engine->moleculeCount(); }

// Current particle positions (framework first, then guest sites in engine order).
uint64_t ref_gcmc_particles(void* h, double* xyz, uint64_t cap) {
    const auto& p = static_cast<RefGcmc*>(h)->engine->particles();
    for (uint64_t i = 0; i < p.size() && i < cap; ++i) {
        xyz[3 * i] = p.x[i];
        xyz[3 * i + 1] = p.y[i];
        xyz[3 * i + 2] = p.z[i];
    }
    return p.size();
}

double ref_gcmc_ewald_energy(void* h) {
    return static_cast<RefGcmc*>(h)->engine->electrostaticEnergyForTesting();
}

double ref_gcmc_ewald_drift(void* h) {
    return static_cast<RefGcmc*>(h)->engine->electrostaticEnergyDriftForTesting();
}

void ref_gcmc_destroy(void* h) { delete static_cast<RefGcmc*>(h); }

// ---------------------------------------------------------------- Peng-Robinson
double ref_pr_fugacity(double tc, double pc, double omega, double t, double p) {
    return engines::PengRobinson({tc, pc, omega}).fugacityPascal(t, p);
}

// readCif: a handle, or NULL with the exception's message in msg
void* ref_read_cif(const char* path, char* msg, size_t cap) {
    try {
        return new io::StructureData(io::readCif(path));
    } catch (const std::exception& e) {
        std::snprintf(msg, cap, "%s", e.what());
        return nullptr;
    }
}
uint64_t ref_structure_size(void* h) { return static_cast<io::StructureData*>(h)->particles.size(); }
uint32_t ref_structure_species(void* h) {
    return (uint32_t) static_cast<io::StructureData*>(h)->speciesSymbols.size();
}
void ref_structure_atoms(void* h, double* m9, double* x, double* y, double* z, double* q,
                         double* mass, uint32_t* sp, double* occ) {
    const auto& s = *static_cast<io::StructureData*>(h);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m9[3 * i + j] = s.lattice.matrix()[i][j];
    for (size_t i = 0; i < s.particles.size(); ++i) {
        x[i] = s.particles.x[i];
        y[i] = s.particles.y[i];
        z[i] = s.particles.z[i];
        q[i] = s.particles.charge[i];
        mass[i] = s.particles.mass[i];
        sp[i] = s.particles.species[i];
        occ[i] = s.occupancy[i];
    }
}
const char* ref_structure_symbol(void* h, uint32_t k) {
    return static_cast<io::StructureData*>(h)->speciesSymbols[k].c_str();
}
const char* ref_structure_label(void* h, uint64_t i) {
    return static_cast<io::StructureData*>(h)->sourceLabel[i].c_str();
}
void ref_structure_free(void* h) { delete static_cast<io::StructureData*>(h); }

// PengRobinsonMixture: 0, or -1 with the exception's message in msg
int ref_pr_mixture(uint32_t n, const double* tc, const double* pc, const double* omega,
                   const double* kij, double t, double p, const double* x, double* z_out,
                   double* f_out, char* msg, size_t cap) {
    try {
        std::vector<engines::PengRobinsonSubstance> subs;
        for (uint32_t i = 0; i < n; ++i) subs.push_back({tc[i], pc[i], omega[i]});
        std::vector<std::vector<double>> k;
        if (kij)
            for (uint32_t i = 0; i < n; ++i) k.emplace_back(kij + (size_t)i * n, kij + (size_t)(i + 1) * n);
        const engines::PengRobinsonMixture eos(std::move(subs), std::move(k));
        const std::vector<double> xs(x, x + n);
        const auto f = eos.fugacitiesPascal(t, p, xs);
        for (uint32_t i = 0; i < n; ++i) f_out[i] = f[i];
        *z_out = eos.compressibilityFactor(t, p, xs);
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(msg, cap, "%s", e.what());
        return -1;
    }
}

}  // extern "C"

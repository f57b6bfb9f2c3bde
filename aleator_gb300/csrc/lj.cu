// LennardJones::computeParticleEnergy (forcefield/pairwise/lennard_jones.cc:158-182)
// for a batch of query particles: one thread per query, ascending j, the
// reference's pairEnergy on the minimum-image distance.
#include <vector>

#include "common.cuh"
#include "grid.cuh"

namespace alea {

namespace {

__global__ void lj_particle_kernel(Lattice L, const double4* __restrict__ p,
                                   const uint32_t* __restrict__ sp, uint64_t n,
                                   const PairParams* __restrict__ table, uint32_t n_species,
                                   double rc, int trunc, const uint64_t* __restrict__ query,
                                   uint64_t nq, const uint64_t* __restrict__ excluded, int nex,
                                   double* __restrict__ out) {
    const uint64_t qi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const uint64_t i = query[qi];
    const double4 a = p[i];
    const PairParams* row = table + (size_t)sp[i] * n_species;
    double e = 0.0;
    for (uint64_t j = 0; j < n; ++j) {
        if (j == i) continue;
        bool skip = false;
        for (int x = 0; x < nex; ++x) skip |= (excluded[x] == j);
        if (skip) continue;
        const double4 b = p[j];
        double dx, dy, dz;
        min_image(L, b.x - a.x, b.y - a.y, b.z - a.z, dx, dy, dz);
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        e += lj_pair_rt(trunc, r, rc, row[sp[j]]);
    }
    out[qi] = e;
}

}  // namespace

void lj_particle_energy(const alea_lennard_jones& lj, const alea_particles& p,
                        const alea_lattice& lat, const uint64_t* query, uint64_t nq,
                        const uint64_t* excluded, uint64_t nex, double* out) {
    require(lj.cutoff > 0.0, ALEA_ERR_INVALID_ARGUMENT, "LennardJones: cutoff must be positive");
    require(lj.n_species > 0, ALEA_ERR_INVALID_ARGUMENT, "LennardJones: no species");
    require(p.n == 0 || (p.x && p.y && p.z), ALEA_ERR_INVALID_ARGUMENT,
            "computeParticleEnergy: particle coordinates missing");
    const Lattice L = make_lattice(lat.m);
    validate_cutoff(L, lj.cutoff, "LennardJones::computeParticleEnergy");
    for (uint64_t i = 0; i < nq; ++i)
        require(query[i] < p.n, ALEA_ERR_OUT_OF_RANGE, "computeParticleEnergy: index out of range");
    for (uint64_t i = 0; i < p.n; ++i)
        require(!p.species || p.species[i] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                "LennardJones::mixedParameters: species out of range");
    require(nex <= 1024, ALEA_ERR_INVALID_ARGUMENT, "computeParticleEnergy: at most 1024 excluded");
    if (nq == 0) return;
    require_device();
    std::vector<double4> packed(p.n);
    std::vector<uint32_t> species(p.n, 0);
    for (uint64_t i = 0; i < p.n; ++i) {
        packed[i] = make_double4(p.x[i], p.y[i], p.z[i], 0.0);
        if (p.species) species[i] = p.species[i];
    }
    std::vector<PairParams> table((size_t)lj.n_species * lj.n_species);
    mixed_table(lj, table.data());
    DevBuf<double4> dp(std::max<size_t>(p.n, 1));
    DevBuf<uint32_t> ds(std::max<size_t>(p.n, 1));
    DevBuf<PairParams> dt(table.size());
    DevBuf<uint64_t> dq(nq), dx(std::max<uint64_t>(nex, 1));
    DevBuf<double> dout(nq);
    dp.upload(packed.data(), p.n);
    ds.upload(species.data(), p.n);
    dt.upload(table.data(), table.size());
    dq.upload(query, nq);
    dx.upload(excluded, nex);
    lj_particle_kernel<<<(unsigned)((nq + 127) / 128), 128>>>(L, dp.p, ds.p, p.n, dt.p,
                                                              lj.n_species, lj.cutoff,
                                                              lj.truncation, dq.p, nq, dx.p,
                                                              (int)nex, dout.p);
    ALEA_CUDA(cudaGetLastError());
    dout.download(out, nq);
    ALEA_CUDA(cudaDeviceSynchronize());
}

}  // namespace alea

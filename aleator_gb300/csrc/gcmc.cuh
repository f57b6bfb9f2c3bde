// GCMC chain state shared by the chain kernel and its host driver.
#pragma once

#include <stdint.h>

namespace alea {

constexpr int GCMC_MAX_SPECIES = 4;  // guest species of one chain (a mixture)

// One chain's scalars (MonteCarloEngine's rng counter, molecule counts,
// fugacities, EwaldIncrementalState's self / exclusion energies and resync
// counter, plus move statistics).
struct ChainState {
    uint64_t seed, stream, call;
    double fugacity[GCMC_MAX_SPECIES];  // K / Å^3 (kPascalToInternal applied), per species
    uint64_t n_mol, n_guest;    // molecules, guest sites
    uint64_t n_of[GCMC_MAX_SPECIES];    // molecules of each species
    uint64_t moves_since_resync, resyncs, steps;
    uint64_t attempted[5], accepted[5];  // translate, rotate, insert, delete, swap
    double sum_n, sum_n2;       // running sums of the molecule count after every move
    double self_e, excl_e;      // committed self and exclusion energies
    double last_du;
    unsigned err;
    unsigned pad;
};

}  // namespace alea

// GCMC chain state shared by the chain kernel and its host driver.
#pragma once

#include <stdint.h>

namespace alea {

// One chain's scalars (MonteCarloEngine's rng counter, molecule count,
// fugacity, EwaldIncrementalState's self / exclusion energies and resync
// counter, plus move statistics).
struct ChainState {
    uint64_t seed, stream, call;
    double fugacity;            // K / Å^3 (kPascalToInternal applied)
    uint64_t n_mol, n_guest;    // molecules, guest sites
    uint64_t moves_since_resync, resyncs, steps;
    uint64_t attempted[4], accepted[4];
    double sum_n, sum_n2;       // running sums of the molecule count after every move
    double self_e, excl_e;      // committed self and exclusion energies
    double last_du;
    unsigned err;
    unsigned pad;
};

}  // namespace alea

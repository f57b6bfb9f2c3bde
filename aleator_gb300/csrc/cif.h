// Internal: the CIF structure reader (cif.cpp).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace alea {

// readCif's StructureData (io/structure_io.hpp:18-40): particles in SoA, the
// cell rows a_i (row-major 3x3), per-species element symbols, and per atom its
// occupancy and the atom_site label it was expanded from.
struct Structure {
    double m[9];
    std::vector<double> x, y, z, charge, mass, occupancy;
    std::vector<uint32_t> species;
    std::vector<std::string> symbols, labels;
};

// Throws Error(ALEA_ERR_RUNTIME) with the reference's CifParseError message.
Structure read_cif(const char* path);

}  // namespace alea

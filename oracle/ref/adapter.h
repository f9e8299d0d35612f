// The drop-in adapter between MolTwister's MD commands and libmtgpu.so (adapter.cpp).
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "mtgpu.h"
#include "MolTwisterState.h"
#include "Cmd/MolTwisterCmdMolDyn/Config/MolDynConfigStruct.h"

namespace mtgpu_adapter {

// The descriptors and the arrays they point to.
struct Descriptors {
    std::vector<double> r, mass, charge;
    std::vector<int32_t> type, mol, nb_count, bonds, angles, dihedrals;
    std::vector<uint8_t> mobile;
    std::vector<std::string> type_names;
    std::vector<mtg_term> nb_terms, bond_terms, angle_terms, dih_terms;
    std::vector<float> nb_tables, bond_tables, angle_tables, dih_tables;
    mtg_system_desc sys{};
    mtg_config_desc cfg{};
};

// Fills d from the state and the `moldyn cfg` settings (reference precision, all-pairs Coulomb,
// the reference's tables); false with a message when a term kind has no counterpart.
bool build(CMolTwisterState* st, const SMolDynConfigStruct& cfg, Descriptors& d, std::string& err);

// `moldyn run` through libmtgpu.so: the descriptors, the reference's initial-state draw (rand()
// seeded with `seed`), numberOfTimeSteps_ steps with the info-line scalars printed every
// outputStride_ steps.  Returns "" or an error message for CCmdRun::lastError_.
std::string run(const SMolDynConfigStruct& cfg, FILE* out, CMolTwisterState* st, uint32_t seed = 1);

}  // namespace mtgpu_adapter

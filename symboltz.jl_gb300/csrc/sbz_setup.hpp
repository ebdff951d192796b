// Host builders for the perturbation-kernel descriptors (see sbz_layout.hpp).
#pragma once
#include <vector>
#include "sbz_layout.hpp"
#include "sbz_background.hpp"

namespace sbz {
int build_model(const sbz_model& m, ModelDesc& M, std::vector<CompDesc>& comps);
int build_cosmo(const Background& B, const ModelDesc& M, const sbz_model& m, CosmoDesc& D);
}  // namespace sbz

// oxg_internal.h - host-side helpers shared between the engine translation units
// (not part of the C ABI).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/oxdna_gb300.h"

namespace oxg {

// Record an error for oxg_last_error() and return `code`.
int internal_set_error(int code, const std::string& msg);
// Host image of a context's FP32 parameter block.
int internal_assemble_block(const oxg_context* c, std::vector<unsigned char>& out);
// Terms that have parameters (bit per term id).
uint32_t internal_present_mask(const oxg_context* c);
// Largest COM cutoff over the terms in `mask` (short-range terms only if short_only).
double internal_max_rcut(const oxg_context* c, uint32_t mask, bool short_only);
// Number of particle / bond types, and whether every bond type has parameters.
int internal_n_types(const oxg_context* c);
bool internal_bonded_complete(const oxg_context* c);
int internal_num_sms();
// Device image (an MlpDev) of a surrogate network, or null.
const void* internal_mlp_device(const oxg_mlp* m);

}  // namespace oxg

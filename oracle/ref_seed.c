/*
 * ref_seed.c -- TEST INFRASTRUCTURE ONLY.
 * Applies the shared seeded perturbation (include/comdgb_seed.h) to a
 * simulation built by the compiled reference.  Kept in its own translation
 * unit because the reference's headers and this library's header declare
 * the same (layout-identical) struct names.
 */
#include "comdgb_seed.h"

void refh_seed_apply_impl(void *s, uint64_t seed, int kind, double amp, double temp_k,
                          double mass_amu) {
  comdgb_seed_apply((simflat_t *)s, seed, kind, amp, temp_k, mass_amu);
}

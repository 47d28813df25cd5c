// transcript.h -- library-internal access to the host Merlin transcript of
// transcript.cpp (the C ABI hp_host_v1_merlin_* wraps the same object).
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/hp_cuda.h"

namespace hp {
void merlin_append(HpMerlinTranscript *t, const char *label, const uint8_t *msg, size_t n);
void merlin_challenge(HpMerlinTranscript *t, const char *label, uint8_t *out, size_t n);
}  // namespace hp

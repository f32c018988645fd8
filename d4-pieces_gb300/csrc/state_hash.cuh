// state_hash.cuh -- hashes and identities of frontier states (device side).
#pragma once

#include "d4e_types.h"

namespace d4e {

// 64-bit finaliser (MurmurHash3 fmix64): a bijection that spreads every
// input bit over the output.
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// Instance-free identity of a state, used as a solve-one parent witness and
// for frontier sampling.  It depends on the state alone, not on the
// instance id or on the table layout, so a solve-one result is the same
// whether the instance runs alone or in a batch.
//   K64  -- the key without its tag (window | used), exact;
//   K128 -- a 64-bit fingerprint of (window, used).
__device__ __forceinline__ unsigned long long witness64(unsigned long long key,
                                                        unsigned long long tag) {
    return key & ~tag;
}
__device__ __forceinline__ unsigned long long witness128(unsigned long long k0,
                                                         unsigned long long k1) {
    return mix64(k0 ^ mix64((k1 & kUsedMask128) ^ 0x2545f4914f6cdd1dull));
}

// Sampling hash of a state identity: a sampled frontier keeps the states
// whose hash is at most a per-instance threshold.
__device__ __forceinline__ unsigned long long sample_hash(unsigned long long wid) {
    return mix64(wid ^ 0x9e3779b97f4a7c15ull);
}

}  // namespace d4e

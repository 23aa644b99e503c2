// Device-side pass program: what the planner uploads for each fused tile pass.
#pragma once

#include <stdint.h>

namespace lsg {

// One fused pass. The tile holds 2^K amplitudes: local bits [0, L) are register bits [0, L)
// (one contiguous run per chunk), local bit L+j is register bit hi[j]. Register bits outside the
// tile (outer[]) enumerate the tiles.
struct PassDesc {
    int K, L, nouter, nops, first_op, pad;
    int hi[32];
    int outer[32];
};

// One operator of a pass, with its bits translated to tile-local positions.
struct TileOp {
    int kind, k;
    int lb[8];      // local bits, most significant first
    int sorted[8];  // the same, ascending
    long long data;    // offset in the pool, complex entries
    long long stride;  // per batch member, complex entries
};

}  // namespace lsg

// Device-side pass program: what the planner uploads for each fused tile pass.
#pragma once

#include <stdint.h>

#include <vector>

namespace lsg {

// One fused pass. The tile holds 2^K amplitudes: local bits [0, L) are register bits [0, L)
// (one contiguous run per chunk), local bit L+j is register bit hi[j]. Register bits outside the
// tile (outer[]) enumerate the tiles.
struct PassDesc {
    int K, L, nouter, nops, first_op, pad;
    int hi[32];
    int outer[32];
};

// Operator kinds beyond the public LSG_OP_* set, used by trajectory programs.
constexpr int kOpMixture = 16;  // per-member branch of a unitary-mixture channel

// One operator of a pass, with its bits translated to tile-local positions.
struct TileOp {
    int kind, k;
    int lb[8];      // local bits, most significant first
    int sorted[8];  // the same, ascending
    long long data;    // offset in the pool, complex entries
    long long stride;  // per batch member, complex entries
    int pred;       // predicate bit the member must have set (0: always set)
    int draw;       // trajectory ops: uniform offset from the member's cursor
    int count;      // mixture branches
    int pad;
};

struct Plan {
    std::vector<PassDesc> passes;
    std::vector<TileOp> ops;
};
// The greedy fusion planner (csrc/engine.cu): lsg_op list -> passes of tile-local operators.
// pred/draw/count (may be null) give trajectory operators their predicate bit, uniform offset and
// branch count.
Plan plan_ops(const struct lsg_op* ops, int nops, int nbits, int K, int L, const int* pred, const int* draw,
              const int* count);

}  // namespace lsg

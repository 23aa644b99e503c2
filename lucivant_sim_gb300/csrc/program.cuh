// Device-side pass program: what the planner uploads for each fused tile pass.
#pragma once

#include <stdint.h>

#ifndef __CUDACC_RTC__
#include <vector>
#endif

namespace lsg {

// One fused pass. The tile holds 2^K amplitudes: local bits [0, L) are register bits [0, L)
// (one contiguous run per chunk), local bit L+j is register bit hi[j]. Register bits outside the
// tile (outer[]) enumerate the tiles.
struct PassDesc {
    int K, L, nouter, nops, first_op, pad;
    int first_block, nblocks;
    int hi[32];
    int outer[32];
    // OR-ed into every tile's base. A run from a basis state skips tiles that are still zero:
    // outer[] then lists only the register bits the earlier passes can have changed, and `fix`
    // holds the basis state's values of the others.
    unsigned long long fix;
    unsigned long long pad2;
};

// A register block: consecutive operators of a pass whose bits together span u <= 4 tile bits.
// Each thread loads groups of 2^u amplitudes into registers once, applies every operator of the
// block with compile-time positions, and stores once. bits[i] is the tile bit of block position i
// (position 0 = most significant bit of the group index); sorted[] the same bits ascending.
// generic = 1: a single operator run by the shared-memory path (wider than a register block).
struct BlockDesc {
    int u, first, nops, generic;
    int bits[4];
    int sorted[4];
    int vec;  // 1, 2 or 4: the block's last positions are tile bits (1,) 0, so each group holds
              // runs of `vec` consecutive elements (vector shared-memory accesses)
    unsigned dep[5];  // group index g -> tile position of its first element: OR of (g << i) & dep[i]
    int pad[2];
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
    int tmpl;       // register-block code: kind and positions (see tile.cuh)
    int pos[8];     // positions of the operator's bits within its block (0 = block MSB)
    int zmask;      // trace-preserving 4x4 operators: coefficients zero for every member
                    // (bit 4 * (row - 1) + column), left out by specialized passes
    int pad;
};

// The descriptors are staged back to back in shared memory, followed by 16-byte operator records:
// each size keeps the next array 16-byte aligned.
static_assert(sizeof(PassDesc) % 16 == 0, "PassDesc keeps 16-byte alignment");
static_assert(sizeof(TileOp) % 16 == 0, "TileOp keeps 16-byte alignment");
static_assert(sizeof(BlockDesc) % 16 == 0, "BlockDesc keeps 16-byte alignment");

#ifndef __CUDACC_RTC__
struct Plan {
    std::vector<PassDesc> passes;
    std::vector<TileOp> ops;
    std::vector<BlockDesc> blocks;
};
#endif

// register-block codes (TileOp::tmpl)
constexpr int kT_DENSE1 = 0;    // + P
constexpr int kT_DENSE2 = 4;    // + 4 * P0 + P1
constexpr int kT_PERM1 = 20;    // + P
constexpr int kT_PERM2 = 24;    // + 4 * P0 + P1
constexpr int kT_DEPOL1 = 40;   // + 4 * Prow + Pcol
constexpr int kT_DEPOL2 = 56;   // canonical positions (row a, row b, col a, col b) = (0, 1, 2, 3)
constexpr int kT_DIAGB = 57;    // diagonal re-indexed by the host in block order: v[e] *= m[e]
constexpr int kT_SCALE = 58;
constexpr int kT_TPD2 = 59;     // + 4 * P0 + P1: real 4x4 transfer matrix whose row 0 is (1,0,0,0)
constexpr int kT_X1 = 75;       // + P: unit-phase X (register swap)
constexpr int kT_CX = 79;       // + 4 * Pcontrol + Ptarget: unit-phase CX (register swap)
constexpr int kT_SWAP = 95;     // + 4 * P0 + P1
constexpr int kT_DENSEB = 111;  // a whole register block as one dense 2^u x 2^u complex matrix (block order)
constexpr int kT_CODES = 112;   // the kernel's codes are exactly 0 .. kT_CODES-1 (a dense switch)
// host-side markers, rewritten before upload: mixtures become dense codes per member in the kernel,
// diagonals become kT_DIAGB
constexpr int kT_MIX1 = 112;    // + P
constexpr int kT_MIX2 = 116;    // + 4 * P0 + P1
constexpr int kT_DIAG = 132;
constexpr int kT_GENERIC = -1;
// The greedy fusion planner (csrc/engine.cu): lsg_op list -> passes of tile-local operators.
// pred/draw/count (may be null) give trajectory operators their predicate bit, uniform offset and
// branch count.
#ifndef __CUDACC_RTC__
Plan plan_ops(const struct lsg_op* ops, int nops, int nbits, int K, int L, const int* pred, const int* draw,
              const int* count, int umax);
#endif

}  // namespace lsg

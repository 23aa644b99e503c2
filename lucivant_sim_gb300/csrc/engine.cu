// Registers and fused gate passes.
//
// lsg_apply replaces Orrery's per-gate full-state sweeps (_apply_slices, engines.py:45-119, and
// the density-matrix updates, engines.py:233-255) with tile passes: the planner groups
// consecutive operators whose bits fit one tile of 2^K amplitudes — the lowest L register bits
// (contiguous, so every copy is a >= 512-byte run) plus up to K-L higher bits chosen per pass
// (qubit-index remapping: a high-qubit gate is brought into the tile by choosing the tile's
// bits, never by transposing the register). Each CTA stages a tile into shared memory with
// cp.async.bulk copies completing on an mbarrier, applies every operator of the pass in shared
// memory, and writes the tile back with bulk stores: one HBM read and one write per pass.
#include <algorithm>
#include <atomic>
#include <complex>
#include <cstring>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "common.cuh"
#include "jit.cuh"
#include "kernels.cuh"
#include "program.cuh"
#include "tile.cuh"

namespace lsg {

// ------------------------------------------------------------------------ errors

static thread_local std::string t_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_error = buf;
    return code;
}

void clear_error() { t_error.clear(); }

static std::mutex g_status_mu;
static int* g_status[64] = {};

int* device_status() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_status_mu);
    if (!g_status[dev]) {
        int* p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return nullptr;
        g_status[dev] = p;
    }
    return g_status[dev];
}

int check_device_status(cudaStream_t stream) {
    int* dev_status = device_status();
    if (!dev_status) return fail(LSG_E_CUDA, "cannot allocate the device status word");
    int status = 0;
    LSG_CUDA(cudaMemcpyAsync(&status, dev_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    LSG_CUDA(cudaStreamSynchronize(stream));
    if (status != 0) {
        cudaMemsetAsync(dev_status, 0, sizeof(int), stream);
        cudaStreamSynchronize(stream);
        return fail(status, "a device-side wait gave up (status %d); the result is not valid", status);
    }
    return LSG_OK;
}

int ensure(Scratch& s, size_t bytes) {
    if (s.bytes >= bytes) return LSG_OK;
    release(s);
    size_t want = std::max<size_t>(bytes, 4096);
    if (s.stream) LSG_CUDA(cudaMallocAsync(&s.ptr, want, s.stream));
    else LSG_CUDA(cudaMalloc(&s.ptr, want));
    s.bytes = want;
    return LSG_OK;
}

void release(Scratch& s) {
    if (s.ptr) {
        if (s.stream) cudaFreeAsync(s.ptr, s.stream);
        else cudaFree(s.ptr);
    }
    s.ptr = nullptr;
    s.bytes = 0;
}

// ------------------------------------------------------------------------ planner

int op_bits_ok(const lsg_op& op, int nbits) {
    if (op.kind == LSG_OP_SCALE) return op.nbits == 0;
    if (op.nbits < 1 || op.nbits > LSG_MAX_OP_BITS) return 0;
    if (op.kind == LSG_OP_MATRIX || op.kind == LSG_OP_PERM || op.kind == kOpMixture) {
        if (op.nbits > 5) return 0;
    } else if (op.kind == LSG_OP_DEPOL) {
        if (op.nbits != 2 && op.nbits != 4) return 0;
    } else if (op.kind != LSG_OP_DIAG) {
        return 0;
    }
    uint64_t seen = 0;
    for (int i = 0; i < op.nbits; ++i) {
        int b = op.bits[i];
        if (b < 0 || b >= nbits || (seen >> b) & 1) return 0;
        seen |= 1ull << b;
    }
    return 1;
}

// Register blocks: consecutive operators of a pass (already in a valid order) grouped while the
// union of their bits stays within umax bits. A two-qubit depolarising operator fixes its block's
// bit order (row a, row b, col a, col b); everything else takes the order of first appearance.
static bool block_kind(const TileOp& t, int umax) {
    switch (t.kind) {
        case LSG_OP_MATRIX: return t.k == 1 || (t.k == 2 && umax >= 2);
        case LSG_OP_PERM: return t.k == 1 || (t.k == 2 && umax >= 2);
        case LSG_OP_DEPOL: return t.k == 2 || (t.k == 4 && umax >= 4);
        case LSG_OP_DIAG: return t.k <= umax;
        case LSG_OP_SCALE: return true;
        case kOpMixture: return t.k == 1 || (t.k == 2 && umax >= 2);
        default: return false;
    }
}

static void finish_block(Plan& plan, int pass_first, int first, int count, std::vector<int>& bits, int depol2,
                         int K, int rb) {
    BlockDesc b{};
    b.first = first - pass_first;  // the kernel indexes the pass's operators from 0
    b.nops = count;
    b.generic = 0;
    std::vector<int> order;
    if (depol2 >= 0) {
        for (int i = 0; i < 4; ++i) order.push_back(plan.ops[depol2].lb[i]);
    } else {
        // dense operators' bits first, in operator order, then the rest in order of appearance:
        // each dense operator takes adjacent positions, so blocks of the same shape (a qubit pair
        // of a Pauli-transfer register, say) run the same few compiled cases
        for (int o = first; o < first + count; ++o) {
            const TileOp& t = plan.ops[o];
            if (t.kind != LSG_OP_MATRIX) continue;
            for (int i = 0; i < t.k; ++i)
                if (std::find(order.begin(), order.end(), t.lb[i]) == order.end()) order.push_back(t.lb[i]);
        }
        for (int b : bits)
            if (std::find(order.begin(), order.end(), b) == order.end()) order.push_back(b);
        // tile bits 1 and 0 go last: a group then holds runs of consecutive elements, read and
        // written with vector shared-memory accesses (which also avoids their bank conflicts)
        for (int low : {1, 0}) {
            auto it = std::find(order.begin(), order.end(), low);
            if (it != order.end()) {
                order.erase(it);
                order.push_back(low);
            }
        }
    }
    // fill up to the register width with the highest unused tile bits: every thread then owns
    // 2^rb amplitudes and the warp's lanes stay on the lowest tile bits
    for (int bit = K - 1; bit >= 0 && (int)order.size() < std::min(rb, K); --bit)
        if (std::find(order.begin(), order.end(), bit) == order.end()) order.push_back(bit);
    if (order.empty()) order.push_back(0);
    b.u = (int)order.size();
    for (int i = 0; i < b.u; ++i) {
        b.bits[i] = order[i];
        b.sorted[i] = order[i];
    }
    std::sort(b.sorted, b.sorted + b.u);
    b.vec = 1;
    if (b.u >= 1 && order[b.u - 1] == 0) b.vec = (b.u >= 2 && order[b.u - 2] == 1) ? 4 : 2;
    // the group index's bits fill the tile bits around the block's: bits of g between the
    // (i-1)-th and i-th block bit (ascending) move up by i
    for (int i = 0; i <= b.u; ++i) {
        const int lo = i == 0 ? 0 : b.sorted[i - 1] + 1;
        const int hi = i == b.u ? K : b.sorted[i];
        unsigned m = 0;
        for (int t = lo; t < hi; ++t) m |= 1u << t;
        b.dep[i] = m;
    }
    for (int i = b.u + 1; i < 5; ++i) b.dep[i] = 0;
    for (int o = first; o < first + count; ++o) {
        TileOp& t = plan.ops[o];
        int P[8] = {0};
        for (int i = 0; i < t.k; ++i)
            for (int j = 0; j < b.u; ++j)
                if (order[j] == t.lb[i]) P[i] = j;
        for (int i = 0; i < 8; ++i) t.pos[i] = P[i];
        switch (t.kind) {
            case LSG_OP_MATRIX: t.tmpl = t.k == 1 ? kT_DENSE1 + P[0] : kT_DENSE2 + 4 * P[0] + P[1]; break;
            case LSG_OP_PERM: t.tmpl = t.k == 1 ? kT_PERM1 + P[0] : kT_PERM2 + 4 * P[0] + P[1]; break;
            case LSG_OP_DEPOL: t.tmpl = t.k == 2 ? kT_DEPOL1 + 4 * P[0] + P[1] : kT_DEPOL2; break;
            case LSG_OP_DIAG: t.tmpl = kT_DIAG; break;
            case LSG_OP_SCALE: t.tmpl = kT_SCALE; break;
            case kOpMixture: t.tmpl = t.k == 1 ? kT_MIX1 + P[0] : kT_MIX2 + 4 * P[0] + P[1]; break;
            default: t.tmpl = kT_GENERIC; break;
        }
    }
    plan.blocks.push_back(b);
}

// Reorder a pass's operators so register blocks come out large: operators on disjoint bits
// commute, so an operator may move ahead of every skipped operator it shares no bit with. Greedy:
// seed a block with the first remaining operator, sweep the rest in program order, and pull in
// each one whose bits keep the block within umax bits and that no skipped operator before it
// touches. Operators keep their program order relative to every operator they share a bit with.
static void reorder_for_blocks(Plan& plan, const PassDesc& pd, int umax) {
    if (umax < 1 || pd.nops < 3) return;
    std::vector<TileOp> in(plan.ops.begin() + pd.first_op, plan.ops.begin() + pd.first_op + pd.nops);
    auto mask_of = [](const TileOp& t) {
        uint64_t m = 0;
        for (int i = 0; i < t.k; ++i) m |= 1ull << t.lb[i];
        return m;
    };
    std::vector<int> rest(in.size());
    for (size_t i = 0; i < in.size(); ++i) rest[i] = (int)i;
    std::vector<TileOp> out;
    out.reserve(in.size());
    while (!rest.empty()) {
        const TileOp& seed = in[rest[0]];
        std::vector<int> take{rest[0]}, left;
        if (!block_kind(seed, umax)) {
            out.push_back(seed);
            rest.erase(rest.begin());
            continue;
        }
        uint64_t bits = mask_of(seed), blocked = 0;
        bool has_d2 = seed.kind == LSG_OP_DEPOL && seed.k == 4;
        for (size_t r = 1; r < rest.size(); ++r) {
            const TileOp& t = in[rest[r]];
            const uint64_t m = mask_of(t);
            bool ok = block_kind(t, umax) && !(m & blocked);
            const uint64_t grown = bits | m;
            const int gsz = __builtin_popcountll(grown);
            const bool d2 = t.kind == LSG_OP_DEPOL && t.k == 4;
            if (ok && gsz > umax) ok = false;
            if (ok && d2 && (has_d2 || gsz != 4)) ok = false;
            if (ok && has_d2 && gsz != 4) ok = false;
            if (ok) {
                take.push_back(rest[r]);
                bits = grown;
                has_d2 = has_d2 || d2;
            } else {
                left.push_back(rest[r]);
                blocked |= m;
            }
        }
        for (int i : take) out.push_back(in[i]);
        rest.swap(left);
    }
    std::copy(out.begin(), out.end(), plan.ops.begin() + pd.first_op);
}

static void form_blocks(Plan& plan, PassDesc& pd, int umax) {
    pd.first_block = (int)plan.blocks.size();
    std::vector<int> bits;
    int start = pd.first_op, count = 0, depol2 = -1;
    auto flush = [&]() {
        if (count) finish_block(plan, pd.first_op, start, count, bits, depol2, pd.K, umax);
        bits.clear();
        count = 0;
        depol2 = -1;
    };
    for (int o = pd.first_op; o < pd.first_op + pd.nops; ++o) {
        TileOp& t = plan.ops[o];
        if (umax < 1 || !block_kind(t, umax)) {
            flush();
            BlockDesc g{};
            g.first = o - pd.first_op;
            g.nops = 1;
            g.generic = 1;
            t.tmpl = kT_GENERIC;
            plan.blocks.push_back(g);
            start = o + 1;
            continue;
        }
        std::vector<int> grown = bits;
        for (int i = 0; i < t.k; ++i)
            if (std::find(grown.begin(), grown.end(), t.lb[i]) == grown.end()) grown.push_back(t.lb[i]);
        const bool is_d2 = t.kind == LSG_OP_DEPOL && t.k == 4;
        bool fits = (int)grown.size() <= umax;
        if (fits && is_d2 && (depol2 >= 0 || (int)grown.size() != 4)) fits = false;
        if (fits && depol2 >= 0 && (int)grown.size() != 4) fits = false;
        if (!fits) {
            flush();
            start = o;
            grown.clear();
            for (int i = 0; i < t.k; ++i) grown.push_back(t.lb[i]);
        }
        bits = grown;
        if (is_d2) depol2 = o;
        ++count;
    }
    flush();
    pd.nblocks = (int)plan.blocks.size() - pd.first_block;
}

// Operators per pass at most: their descriptors are staged in shared memory beside the tile
// (192 x 136 B + blocks stays under 40 KB, so two pipelined CTAs still share an SM).
constexpr int kMaxPassOps = 192;

// Plan and launch choices for the program being created on this thread (lsg_program_create_opts);
// zero fields keep the defaults (and their environment knobs).
struct PlanChoice {
    int tile_bits = 0, low_bits = 0, ctas = 0, max_ops = 0;
};
static thread_local PlanChoice t_choice;

// Starting tiles the planner tries per pass (LSG_PLAN_SEEDS; 1 = the plain greedy sweep). More
// than about 64 found no better plan for brickwork circuits of 12-20 qubits.
static int plan_seeds() {
    const char* env = getenv("LSG_PLAN_SEEDS");
    return env ? std::max(1, atoi(env)) : 64;
}

// Greedy fusion: sweep the remaining operators; an operator joins the current pass when its bits
// fit the tile, the pass has room, and no operator deferred earlier in the sweep shares a bit with
// it (so program order is kept wherever it matters). Deferred operators start the next sweep.
// Each pass tries several starting tiles and keeps the sweep that takes the most operators.
Plan plan_ops(const lsg_op* ops, int nops, int nbits, int K, int L, const int* pred, const int* draw,
              const int* count, int umax) {
    Plan plan;
    std::vector<int> remaining(nops);
    for (int i = 0; i < nops; ++i) remaining[i] = i;
    const uint64_t low = (L >= 64) ? ~0ull : ((1ull << L) - 1);
    auto op_mask = [&](int idx) {
        uint64_t mask = 0;
        for (int i = 0; i < ops[idx].nbits; ++i) mask |= 1ull << ops[idx].bits[i];
        return mask;
    };
    const char* ops_env = getenv("LSG_PASS_OPS");
    const int max_ops = t_choice.max_ops ? std::max(1, std::min(kMaxPassOps, t_choice.max_ops))
                        : ops_env        ? std::max(1, std::min(kMaxPassOps, atoi(ops_env)))
                                         : kMaxPassOps;
    // One pass by the greedy sweep from a starting tile: an operator joins when its bits fit and no
    // operator deferred earlier in the sweep shares a bit with it (program order where it matters).
    std::vector<uint64_t> masks(nops);
    bool scalar_ops = false;  // operators on no bits (global phases) join any sweep at any point
    for (int i = 0; i < nops; ++i) {
        masks[i] = op_mask(i);
        scalar_ops = scalar_ops || masks[i] == 0;
    }
    const uint64_t all = nbits >= 64 ? ~0ull : ((1ull << nbits) - 1);
    // A sweep stops early once every register bit is blocked: no later operator can join. The
    // operators from `*stop` on are then deferred as they stand.
    auto sweep = [&](uint64_t start, uint64_t* tile_out, std::vector<int>* taken, std::vector<int>* deferred,
                     size_t* stop) {
        uint64_t tile = start, blocked = 0;
        taken->clear();
        deferred->clear();
        size_t i = 0;
        for (; i < remaining.size(); ++i) {
            if (blocked == all && !scalar_ops) break;
            const int idx = remaining[i];
            const uint64_t mask = masks[idx];
            if ((mask & blocked) || (int)taken->size() >= max_ops) {
                deferred->push_back(idx);
                blocked |= mask;
                continue;
            }
            const uint64_t grown = tile | mask;
            if (__builtin_popcountll(grown) <= K) {
                tile = grown;
                taken->push_back(idx);
            } else {
                deferred->push_back(idx);
                blocked |= mask;
            }
        }
        *stop = i;
        *tile_out = tile;
    };
    const int seeds = plan_seeds();
    while (!remaining.empty()) {
        uint64_t tile = low;
        std::vector<int> taken, deferred;
        size_t stop = 0;
        sweep(low, &tile, &taken, &deferred, &stop);
        // Other starting tiles: the low bits plus the bits of one of the next operators, so the tile
        // can form around later work instead of the first operators' bits; the sweep that takes the
        // most operators wins (the first one on ties).
        std::vector<int> t2, d2;
        for (int j = 1; j < seeds && j < (int)remaining.size(); ++j) {
            uint64_t start = low | masks[remaining[j]];
            if (__builtin_popcountll(start) > K) continue;
            uint64_t tile2;
            size_t stop2 = 0;
            sweep(start, &tile2, &t2, &d2, &stop2);
            if (t2.size() > taken.size()) {
                tile = tile2;
                taken.swap(t2);
                deferred.swap(d2);
                stop = stop2;
            }
        }
        deferred.insert(deferred.end(), remaining.begin() + (std::ptrdiff_t)stop, remaining.end());
        if (taken.empty()) {  // an operator wider than the tile allows: no progress possible
            plan.passes.clear();
            plan.ops.clear();
            return plan;
        }
        // fill the tile up to K bits with the lowest unused bits (wider contiguous chunks)
        for (int b = 0; b < nbits && __builtin_popcountll(tile) < K; ++b) tile |= 1ull << b;
        PassDesc pd{};
        pd.K = K;
        int l = 0;
        while (l < nbits && ((tile >> l) & 1)) ++l;
        pd.L = std::min(l, K);
        int nhi = 0, nout = 0;
        int local_of[64];
        for (int b = 0; b < nbits; ++b) {
            if ((tile >> b) & 1) {
                if (b < pd.L) {
                    local_of[b] = b;
                } else {
                    local_of[b] = pd.L + nhi;
                    pd.hi[nhi++] = b;
                }
            } else {
                pd.outer[nout++] = b;
            }
        }
        pd.nouter = nout;
        pd.first_op = (int)plan.ops.size();
        pd.nops = (int)taken.size();
        for (int idx : taken) {
            const lsg_op& op = ops[idx];
            TileOp t{};
            t.kind = op.kind;
            t.k = op.nbits;
            for (int i = 0; i < op.nbits; ++i) {
                t.lb[i] = local_of[op.bits[i]];
                t.sorted[i] = t.lb[i];
            }
            std::sort(t.sorted, t.sorted + op.nbits);
            t.data = op.data;
            t.stride = op.batch_stride;
            t.pred = pred ? pred[idx] : 0;
            t.draw = draw ? draw[idx] : 0;
            t.count = count ? count[idx] : 0;
            plan.ops.push_back(t);
        }
        reorder_for_blocks(plan, pd, umax);
        form_blocks(plan, pd, umax);
        plan.passes.push_back(pd);
        remaining.swap(deferred);
    }
    return plan;
}

// Widest register block: 16 elements per thread for 4- and 8-byte elements, 8 complex128.
int block_bits_for(int precision) {
    const int top = lsg_elem_bytes(precision) == 16 ? 3 : 4;
    int u = top;
    if (const char* env = getenv("LSG_BLOCK_BITS")) u = atoi(env);
    return std::max(0, std::min(u, top));
}

static Plan plan_passes(const lsg_op* ops, int nops, int nbits, int K, int L, int umax) {
    return plan_ops(ops, nops, nbits, K, L, nullptr, nullptr, nullptr, umax);
}

// ------------------------------------------------------------------------ programs

// Every block indexes inside its pass's operators and covers them exactly; every operator bit
// lies inside its tile; every tile bit is a register bit.
static int check_plan(const Plan& plan) {
    for (const PassDesc& pd : plan.passes) {
        int covered = 0;
        for (int bi = pd.first_block; bi < pd.first_block + pd.nblocks; ++bi) {
            if (bi < 0 || bi >= (int)plan.blocks.size()) return fail(LSG_E_ARG, "internal planning error: block index");
            const BlockDesc& b = plan.blocks[bi];
            if (b.first != covered || b.nops < 1 || b.first + b.nops > pd.nops || b.generic < 0 || b.generic > 1 ||
                (!b.generic && (b.u < 1 || b.u > 4)))
                return fail(LSG_E_ARG, "internal planning error: a block outside its pass");
            for (int i = 0; !b.generic && i < b.u; ++i)
                if (b.bits[i] < 0 || b.bits[i] >= pd.K) return fail(LSG_E_ARG, "internal planning error: block bit");
            if (!b.generic) {  // the deposit masks place every group index where the insertion chain does
                const uint32_t groups = 1u << (pd.K - b.u);
                for (uint32_t g0 : {0u, 1u, groups / 2 + 1, groups - 1, 0x55555555u, 0xAAAAAAAAu}) {
                    const uint32_t g = g0 & (groups - 1);
                    uint32_t want = g, got = 0;
                    for (int i = 0; i < b.u; ++i) {
                        const int sb = b.sorted[i];
                        want = ((want >> sb) << (sb + 1)) | (want & ((1u << sb) - 1));
                    }
                    for (int i = 0; i <= b.u; ++i) got |= (g << i) & b.dep[i];
                    if (got != want) return fail(LSG_E_ARG, "internal planning error: block deposit masks");
                    if (b.vec > 1 && (got & (uint32_t)(b.vec - 1)))
                        return fail(LSG_E_ARG, "internal planning error: vector access misaligned");
                }
            }
            covered += b.nops;
        }
        if (covered != pd.nops) return fail(LSG_E_ARG, "internal planning error: blocks do not cover the pass");
        for (int o = pd.first_op; o < pd.first_op + pd.nops; ++o) {
            const TileOp& t = plan.ops[o];
            for (int i = 0; i < t.k; ++i)
                if (t.lb[i] < 0 || t.lb[i] >= pd.K) return fail(LSG_E_ARG, "internal planning error: operator bit");
        }
        if (pd.L < 0 || pd.L > pd.K || pd.nouter < 0) return fail(LSG_E_ARG, "internal planning error: tile shape");
    }
    return LSG_OK;
}

// Tile bits: 32 KB tiles of complex64 or real64 (2^12), 2^11 complex128, 2^13 real32.
int tile_bits_for(int nbits, int precision) {
    const size_t eb = lsg_elem_bytes(precision);
    int K = eb == 16 ? 11 : eb == 8 ? 12 : 13;
    if (t_choice.tile_bits) K = t_choice.tile_bits;
    else if (const char* env = getenv("LSG_TILE_BITS")) K = atoi(env);
    return std::max(0, std::min(K, nbits));
}

// Register bits every tile keeps: 2^L contiguous elements, 512 bytes per copy (smaller copies
// leave HBM well below its streaming rate: a real32 pass with 256-byte copies took twice as long
// as the same work with 512-byte copies).
int low_bits_for(int nbits, int precision) {
    const size_t eb = lsg_elem_bytes(precision);
    int L = eb == 16 ? 5 : eb == 8 ? 6 : 7;
    if (t_choice.low_bits) L = t_choice.low_bits;
    else if (const char* env = getenv("LSG_LOW_BITS")) L = atoi(env);
    return std::max(0, std::min(L, nbits));
}

static int validate_ops(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops,
                        const double* pool, int64_t pool_entries) {
    if (nops < 0 || (nops > 0 && !ops) || pool_entries < 0 || (pool_entries > 0 && !pool))
        return fail(LSG_E_ARG, "bad operator list or pool");
    const bool real = lsg_precision_real(precision);
    if (real) {  // Pauli-transfer registers: real matrices only, channels already in transfer form
        for (int i = 0; i < nops; ++i)
            if (ops[i].kind == LSG_OP_DEPOL)
                return fail(LSG_E_ARG, "operator %d: a real register takes depolarising channels as DIAG operators", i);
        for (int64_t i = 0; i < pool_entries; ++i)
            if (pool[2 * i + 1] != 0.0) return fail(LSG_E_ARG, "a real register takes real operator data only");
    }
    for (int i = 0; i < nops; ++i) {
        const lsg_op& op = ops[i];
        if (!op_bits_ok(op, nbits)) return fail(LSG_E_ARG, "operator %d has a bad kind or bits", i);
        int64_t need = 1;
        const int64_t d = 1ll << (op.kind == LSG_OP_DEPOL ? 0 : op.nbits);
        if (op.kind == LSG_OP_MATRIX) need = d * d;
        else if (op.kind == LSG_OP_DIAG) need = d;
        else if (op.kind == LSG_OP_PERM) need = 2 * d;
        const int64_t last = op.data + need + (batch - 1) * op.batch_stride;
        if (op.data < 0 || op.batch_stride < 0 || last > pool_entries)
            return fail(LSG_E_ARG, "operator %d reads outside the pool", i);
        if (op.kind == LSG_OP_PERM) {
            for (int64_t b = 0; b < batch; ++b)
                for (int64_t r = 0; r < d; ++r) {
                    const double src = pool[2 * (op.data + b * op.batch_stride + d + r)];
                    if (!(src >= 0 && src < (double)d) || src != (double)(int64_t)src)
                        return fail(LSG_E_ARG, "operator %d has a bad permutation", i);
                }
        }
    }
    return LSG_OK;
}

}  // namespace lsg

// A planned and uploaded operator list: the passes, their operators and the data pool in the
// register precision, resident on the device, ready to launch on any register of the same shape.
struct lsg_program_s {
    int nbits = 0, precision = 0;
    int64_t batch = 1;
    lsg::Plan plan;
    lsg::Scratch dev;
    size_t head_aligned = 0;
    size_t smem = 0;
    int K = 0;
    std::vector<cudaEvent_t> events;
    std::shared_ptr<lsg::JitPasses> jit;  // specialized passes, when the program could be specialized
    // runs from a basis state: the passes restricted to tiles that can be nonzero (uploaded after
    // the block descriptors, for the basis index `basis_index`)
    std::vector<lsg::PassDesc> basis_passes;
    int64_t basis_index = -1;
    size_t basis_off = 0;
    // the pool section (caller's pool, then relocated and fused data) in the register precision:
    // kept by host-only builds, whose data a program of the same structure takes over
    std::vector<unsigned char> pool_bytes;
    lsg::PlanChoice choice;  // the plan choices it was made with
    // the operator table and the plan before lowering: a template's new data is lowered onto this
    // plan without planning again (lsg_program_set_data)
    std::vector<lsg_op> src_ops;
    lsg::Plan raw_plan;
    // the template's CUDA graph: set basis state + every pass, captured for one register and index
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_uid = 0;
    int64_t graph_index = -1;
};

namespace lsg {

// Let a kernel take all the dynamic shared memory the device allows, once per kernel and
// device (the attribute is global to the function: setting it per launch would race between
// threads launching the same kernel with different sizes).
static std::mutex g_smem_mu;
static std::set<std::pair<const void*, int>> g_smem_done;  // (kernel, device) pairs already raised

template <typename K>
static int allow_smem(K kern) {
    int dev = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_smem_mu);
    const auto key = std::make_pair(reinterpret_cast<const void*>(kern), dev);
    if (g_smem_done.count(key)) return LSG_OK;
    int optin = 0;
    LSG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    LSG_CUDA(cudaFuncGetAttributes(&fa, kern));
    LSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    g_smem_done.insert(key);
    return LSG_OK;
}

template <typename T>
static int launch_passes(lsg_program_s* p, lsg_state_s* s, cudaEvent_t* marks, const TrajCtx& ctx, bool from_basis) {
    const size_t tile_bytes = sizeof(T) << p->K;
    const size_t meta = p->smem - tile_bytes;
    const int L = p->plan.passes.empty() ? 0 : p->plan.passes[0].L;
    const bool bulk = ((sizeof(T) << L) % 16) == 0;
    const bool pipe = bulk && getenv("LSG_NO_PIPELINE") == nullptr && 2 * tile_bytes + meta <= 200 * 1024;
    // the passes as launched: all tiles, or (from a basis state) the tiles that can be nonzero
    const std::vector<PassDesc>& host_pd = from_basis ? p->basis_passes : p->plan.passes;
    std::vector<int64_t> tpm(host_pd.size());
    for (size_t i = 0; i < host_pd.size(); ++i) tpm[i] = 1ll << host_pd[i].nouter;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int* status = device_status();
    if (!status) return fail(LSG_E_CUDA, "cannot allocate the device status word");
    const PassDesc* plan_pd_dev = reinterpret_cast<const PassDesc*>(p->dev.ptr);
    const TileOp* ops_dev = reinterpret_cast<const TileOp*>(plan_pd_dev + p->plan.passes.size());
    const BlockDesc* blk_dev = reinterpret_cast<const BlockDesc*>(ops_dev + p->plan.ops.size());
    const PassDesc* pd_dev =
        from_basis ? reinterpret_cast<const PassDesc*>(static_cast<unsigned char*>(p->dev.ptr) + p->basis_off) : plan_pd_dev;
    const T* pool_dev = reinterpret_cast<const T*>(static_cast<unsigned char*>(p->dev.ptr) + p->head_aligned);
    T* state = reinterpret_cast<T*>(s->data);
    if (p->jit && bulk && ctx.u == nullptr) {
        LSG_CHECK(jit_launch(*p->jit, p->plan, state, s->elems, pd_dev, sizeof(PassDesc), pool_dev, tpm, s->batch, status,
                             tile_bytes, s->stream, marks));
        if (marks) LSG_CUDA(cudaEventRecord(marks[p->plan.passes.size()], s->stream));
        return LSG_OK;
    }
    if (pipe) {
        // each pass gets the shared memory its own operators need: short passes fit more CTAs per SM
        const void* kern = PassKernels<T>::pipe();
        LSG_CHECK(allow_smem(kern));
        size_t last_smem = 0;
        int64_t grid = 1;
        for (size_t i = 0; i < p->plan.passes.size(); ++i) {
            const PassDesc& pd = p->plan.passes[i];
            const int64_t total = tpm[i] * s->batch;
            const size_t smem = 2 * tile_bytes + (size_t)pd.nops * (sizeof(TileOp) + 16) + (size_t)pd.nblocks * sizeof(BlockDesc);
            if (smem != last_smem) {
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPipeThreads, smem);
                last_smem = smem;
            }
            grid = std::max<int64_t>(1, std::min<int64_t>(total, (int64_t)sms * std::max(per_sm, 1)));
            if (marks) LSG_CUDA(cudaEventRecord(marks[i], s->stream));
            PassKernels<T>::launch_pipe((unsigned)grid, smem, s->stream, state, s->elems, pd_dev + i, ops_dev, blk_dev,
                                        pool_dev, tpm[i], total, status, ctx);
        }
    } else {
        const void* kern = PassKernels<T>::pass();
        LSG_CHECK(allow_smem(kern));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, p->smem);
        for (size_t i = 0; i < p->plan.passes.size(); ++i) {
            const int64_t total = tpm[i] * s->batch;
            const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(total, (int64_t)sms * std::max(per_sm, 1) * 4));
            if (marks) LSG_CUDA(cudaEventRecord(marks[i], s->stream));
            PassKernels<T>::launch_pass((unsigned)grid, p->smem, s->stream, state, s->elems, pd_dev + i, ops_dev, blk_dev,
                                        pool_dev, tpm[i], total, status, ctx);
        }
    }
    if (marks) LSG_CUDA(cudaEventRecord(marks[p->plan.passes.size()], s->stream));
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

// The passes of a run that starts from basis state `index` (lsg_state_set_basis), restricted to
// the tiles that can be nonzero. A basis state fixes register bits: every bit of a complex
// register (the amplitude index), the Pauli x digits of a real Pauli-transfer register (bits
// n..2n-1 are 0; its z digits are free). An operator that is not diagonal frees its bits for the
// passes after it; a diagonal one keeps them. Tiles of pass p whose outer bits differ from the
// fixed values hold zeros and pass p's operators (acting on tile bits only) keep them zero, so pass
// p enumerates the free outer bits only and ORs the fixed values into every tile's base.
static std::vector<PassDesc> basis_passes(const Plan& plan, int nbits, int precision, int64_t index) {
    const bool real = lsg_precision_real(precision);
    uint64_t fixed = nbits >= 64 ? ~0ull : ((1ull << nbits) - 1);
    uint64_t value = real ? 0 : (uint64_t)index;
    if (real) fixed &= ~((1ull << (nbits / 2)) - 1);  // z digits are free
    std::vector<PassDesc> out(plan.passes.begin(), plan.passes.end());
    for (size_t i = 0; i < out.size(); ++i) {
        PassDesc& pd = out[i];
        const PassDesc& src = plan.passes[i];
        pd.nouter = 0;
        pd.fix = 0;
        for (int j = 0; j < src.nouter; ++j) {
            const int bit = src.outer[j];
            if ((fixed >> bit) & 1) pd.fix |= value & (1ull << bit);
            else pd.outer[pd.nouter++] = bit;
        }
        for (int j = pd.nouter; j < 32; ++j) pd.outer[j] = 0;
        for (int o = src.first_op; o < src.first_op + src.nops; ++o) {
            const TileOp& t = plan.ops[o];
            if (t.kind == LSG_OP_DIAG || t.kind == LSG_OP_SCALE) continue;
            for (int k = 0; k < t.k; ++k) {
                const int lb = t.lb[k];
                const int reg = lb < src.L ? lb : src.hi[lb - src.L];
                fixed &= ~(1ull << reg);
            }
        }
    }
    return out;
}

// ---- whole-block fusion (complex registers): a register block whose operators cost more than one
// dense 2^u x 2^u product becomes that product, formed in FP64 on the host and rounded once.

// The block operators a fused block may hold: unconditional unitary pieces (dense, permutation,
// diagonal, scale) of complex registers.
static bool block_fusable_op(const TileOp& t) {
    if (t.pred != 0) return false;
    const int c = t.tmpl;
    return (c >= kT_DENSE1 && c < kT_DENSE2 + 16) || (c >= kT_PERM1 && c < kT_PERM2 + 16) || c == kT_SCALE ||
           c == kT_DIAG || (c >= kT_X1 && c < kT_SWAP + 16);
}

// Per-element work of a block operator in complex multiply-add units (a dense 1-bit operator is
// two per element), plus the interpreter's cost of taking one operator: about a quarter of the
// work of a dense 1-bit operator for complex64 registers, whose passes are bound by instruction
// issue, and little for complex128 ones, bound by FP64 arithmetic.
static double block_op_cost(const TileOp& t, double overhead) {
    const int c = t.tmpl;
    double work = 1.0;  // phased permutation, diagonal, scale: one complex product
    if (c >= kT_DENSE1 && c < kT_DENSE1 + 4) work = 2.0;
    else if (c >= kT_DENSE2 && c < kT_DENSE2 + 16) work = 4.0;
    else if ((c >= kT_X1 && c < kT_X1 + 4) || (c >= kT_CX && c < kT_CX + 16) || (c >= kT_SWAP && c < kT_SWAP + 16)) work = 0.25;
    return work + overhead;
}

// One operator on a block's 2^U amplitudes (block order: position P is group bit U-1-P), by the
// operator kind's own definition (lsg.h), in FP64.
static void host_block_op(std::complex<double>* v, int U, const TileOp& t, const double* pool, int64_t member) {
    const double* m = pool + 2 * (t.data + member * t.stride);
    auto cx = [&](int i) { return std::complex<double>(m[2 * i], m[2 * i + 1]); };
    const int D = 1 << U;
    if (t.kind == LSG_OP_SCALE) {
        for (int e = 0; e < D; ++e) v[e] *= cx(0);
        return;
    }
    const int k = t.k, d = 1 << k;
    uint32_t dep[5] = {0, 0, 0, 0, 0}, mask = 0;
    for (int i = 0; i < k; ++i) {
        dep[i] = 1u << (U - 1 - t.pos[i]);
        mask |= dep[i];
    }
    auto at = [&](int e, int c) {
        uint32_t a = (uint32_t)e;
        for (int i = 0; i < k; ++i)
            if ((c >> (k - 1 - i)) & 1) a |= dep[i];
        return a;
    };
    std::complex<double> a[32], o[32];
    for (int e = 0; e < D; ++e) {
        if ((uint32_t)e & mask) continue;
        for (int c = 0; c < d; ++c) a[c] = v[at(e, c)];
        for (int r = 0; r < d; ++r) {
            if (t.kind == LSG_OP_MATRIX) {
                std::complex<double> acc = 0.0;
                for (int c = 0; c < d; ++c) acc += cx(r * d + c) * a[c];
                o[r] = acc;
            } else if (t.kind == LSG_OP_PERM) {
                o[r] = cx(r) * a[(int)m[2 * (d + r)] & (d - 1)];
            } else {
                o[r] = cx(r) * a[r];
            }
        }
        for (int r = 0; r < d; ++r) v[at(e, r)] = o[r];
    }
}

// Plan and lower `ops`; with `upload`, copy the program to the device (otherwise only the host
// plan is made: no device call).
static int program_build(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops, const double* pool,
                         int64_t pool_entries, const int* pred, const int* draw, const int* count, lsg_program_s** out,
                         cudaStream_t stream, bool upload, const Plan* preplanned = nullptr) {
    auto* p = new lsg_program_s();
    p->nbits = nbits;
    p->precision = precision;
    p->batch = batch;
    p->choice = t_choice;
    p->dev.stream = stream;
    p->K = tile_bits_for(nbits, precision);
    const int L = std::min(p->K, low_bits_for(nbits, precision));
    if (nops > 0) {
        p->plan = preplanned ? *preplanned : plan_ops(ops, nops, nbits, p->K, L, pred, draw, count, block_bits_for(precision));
        if (upload && !pred && !draw && !count) {
            p->src_ops.assign(ops, ops + nops);
            p->raw_plan = p->plan;
        }
        if (p->plan.passes.empty()) {
            delete p;
            return fail(LSG_E_ARG, "an operator does not fit a tile of %d bits (%d kept low)", tile_bits_for(nbits, precision), L);
        }
    }
    if (check_plan(p->plan) != LSG_OK) {
        delete p;
        return LSG_E_ARG;
    }
    // real (Pauli-transfer) 4x4 operators whose first row is (1,0,0,0) for every member: trace
    // preserving; the kernel skips that row
    if (lsg_precision_real(precision))
        for (TileOp& t : p->plan.ops) {
            if (t.kind != LSG_OP_MATRIX || t.k != 2 || t.tmpl < kT_DENSE2 || t.tmpl >= kT_DENSE2 + 16) continue;
            bool tp = true;
            for (int64_t b = 0; b < (t.stride ? batch : 1) && tp; ++b)
                for (int c = 0; c < 4 && tp; ++c) tp = pool[2 * (t.data + b * t.stride + c)] == (c == 0 ? 1.0 : 0.0);
            if (!tp) continue;
            t.tmpl = kT_TPD2 + (t.tmpl - kT_DENSE2);
            int zmask = (1 << 12) - 1;  // rows 1-3: the coefficients that are zero for every member
            for (int64_t b = 0; b < (t.stride ? batch : 1) && zmask; ++b)
                for (int i = 0; i < 12; ++i)
                    if (pool[2 * (t.data + b * t.stride + 4 + i)] != 0.0) zmask &= ~(1 << i);
            t.zmask = zmask;
        }
    // permutations with unit phases shared by all members are register renames
    for (TileOp& t : p->plan.ops) {
        if (t.kind != LSG_OP_PERM || t.stride != 0 || t.tmpl == kT_GENERIC) continue;
        const int d = 1 << t.k;
        bool unit = true;
        int src[4] = {0, 0, 0, 0};
        for (int r = 0; r < d && unit; ++r) {
            unit = pool[2 * (t.data + r)] == 1.0 && pool[2 * (t.data + r) + 1] == 0.0;
            src[r] = (int)pool[2 * (t.data + d + r)];
        }
        if (!unit) continue;
        if (t.k == 1 && src[0] == 1 && src[1] == 0) t.tmpl = kT_X1 + t.pos[0];
        if (t.k == 2) {
            const int P0 = t.pos[0], P1 = t.pos[1];
            if (src[0] == 0 && src[1] == 1 && src[2] == 3 && src[3] == 2) t.tmpl = kT_CX + 4 * P0 + P1;  // first controls
            else if (src[0] == 0 && src[1] == 3 && src[2] == 2 && src[3] == 1) t.tmpl = kT_CX + 4 * P1 + P0;
            else if (src[0] == 0 && src[1] == 2 && src[2] == 1 && src[3] == 3) t.tmpl = kT_SWAP + 4 * P0 + P1;
        }
    }
    // Register-block operator data, copied once here into an extension of the pool: diagonals
    // re-indexed in block order (the kernel multiplies v[e] by m[e] with no index arithmetic), and
    // dense matrices, diagonals and mixture matrices placed on 16-byte boundaries (the kernel reads
    // them with 16-byte loads), per member when the data differs per member.
    std::vector<double> ext;
    ext.reserve((size_t)(2 * pool_entries + pool_entries) + 4096);  // relocated data: about the pool again
    const int64_t per = 16 / (int64_t)lsg_elem_bytes(precision);  // entries per 16 bytes
    auto round_up = [&](int64_t x) { return (x + per - 1) / per * per; };
    auto pad_ext = [&](int64_t lead) {  // pad so that entry (end + lead) is 16-byte aligned
        while ((pool_entries + (int64_t)ext.size() / 2 + lead) % per) {
            ext.push_back(0.0);
            ext.push_back(0.0);
        }
    };
    const char* fuse_env = getenv("LSG_FUSE_BLOCKS");
    const bool fuse = !lsg_precision_real(precision) && !(fuse_env && fuse_env[0] == '0');
    for (const PassDesc& pd : p->plan.passes)
        for (int bi = pd.first_block; bi < pd.first_block + pd.nblocks; ++bi) {
            BlockDesc& blk = p->plan.blocks[bi];
            if (blk.generic) continue;
            if (fuse && blk.u >= 2 && blk.nops > 1) {
                const int U = blk.u, D = 1 << U;
                const double overhead = precision == LSG_C64 ? 0.5 : 0.1;
                bool ok = true;
                bool per_member = false;
                double cost = 0.0;
                for (int o = blk.first; o < blk.first + blk.nops && ok; ++o) {
                    const TileOp& t = p->plan.ops[pd.first_op + o];
                    ok = block_fusable_op(t);
                    per_member |= t.stride != 0;
                    cost += block_op_cost(t, overhead);
                }
                // one dense block: D complex multiply-adds per element, its rows read per group
                if (ok && cost > 1.1 * ((double)D + overhead + (double)D / 16.0)) {
                    const int64_t members = per_member ? batch : 1;
                    const int64_t len = (int64_t)D * D;
                    pad_ext(0);
                    const int64_t at = pool_entries + (int64_t)ext.size() / 2;
                    std::vector<std::complex<double>> col(D);
                    std::vector<double> mat((size_t)2 * len);
                    for (int64_t b = 0; b < members; ++b) {
                        for (int c = 0; c < D; ++c) {
                            std::fill(col.begin(), col.end(), std::complex<double>(0.0, 0.0));
                            col[c] = 1.0;
                            for (int o = blk.first; o < blk.first + blk.nops; ++o) {
                                const TileOp& t = p->plan.ops[pd.first_op + o];
                                host_block_op(col.data(), U, t, pool, t.stride ? b : 0);
                            }
                            for (int r = 0; r < D; ++r) {
                                mat[2 * ((size_t)r * D + c)] = col[r].real();
                                mat[2 * ((size_t)r * D + c) + 1] = col[r].imag();
                            }
                        }
                        ext.insert(ext.end(), mat.begin(), mat.end());
                        ext.resize(ext.size() + 2 * (size_t)(round_up(len) - len), 0.0);
                    }
                    TileOp& f = p->plan.ops[pd.first_op + blk.first];
                    f.kind = LSG_OP_MATRIX;
                    f.k = U;
                    for (int i = 0; i < 8; ++i) {
                        f.lb[i] = i < U ? blk.bits[i] : 0;
                        f.sorted[i] = i < U ? blk.sorted[i] : 0;
                        f.pos[i] = i < U ? i : 0;
                    }
                    f.data = at;
                    f.stride = members > 1 ? round_up(len) : 0;
                    f.tmpl = kT_DENSEB;
                    f.zmask = 0;
                    blk.nops = 1;
                    continue;
                }
            }
            for (int o = blk.first; o < blk.first + blk.nops; ++o) {
                TileOp& t = p->plan.ops[pd.first_op + o];
                const int64_t members = t.stride ? batch : 1;
                if (t.tmpl == kT_DIAG) {
                    const int u = blk.u, d = 1 << u;
                    const int64_t stride = round_up(d);
                    pad_ext(0);
                    const int64_t at = pool_entries + (int64_t)ext.size() / 2;
                    for (int64_t b = 0; b < members; ++b) {
                        for (int e = 0; e < d; ++e) {
                            int j = 0;
                            for (int i = 0; i < t.k; ++i) j = (j << 1) | ((e >> (u - 1 - t.pos[i])) & 1);
                            const int64_t src = t.data + b * t.stride + j;
                            ext.push_back(pool[2 * src]);
                            ext.push_back(pool[2 * src + 1]);
                        }
                        for (int64_t e = d; e < stride; ++e) {
                            ext.push_back(0.0);
                            ext.push_back(0.0);
                        }
                    }
                    t.data = at;
                    t.stride = t.stride ? stride : 0;
                    t.tmpl = kT_DIAGB;
                    continue;
                }
                const bool dense = (t.tmpl >= kT_DENSE1 && t.tmpl < kT_DENSE2 + 16) || (t.tmpl >= kT_TPD2 && t.tmpl < kT_TPD2 + 16);
                const bool mix = t.tmpl >= kT_MIX1 && t.tmpl < kT_MIX2 + 16;
                if (!dense && !mix) continue;
                const int64_t d = 1ll << t.k;
                const int64_t lead = mix ? t.count : 0;  // a mixture's branch table precedes its matrices
                const int64_t len = mix ? t.count + t.count * d * d : d * d;
                const int64_t stride = round_up(len);
                pad_ext(lead);
                const int64_t at = pool_entries + (int64_t)ext.size() / 2;
                for (int64_t b = 0; b < members; ++b) {
                    const double* src = pool + 2 * (t.data + b * t.stride);
                    ext.insert(ext.end(), src, src + 2 * len);
                    ext.resize(ext.size() + 2 * (stride - len), 0.0);
                }
                t.data = at;
                t.stride = t.stride ? stride : 0;
            }
        }
    // every register-block operator now carries a kernel code (mixtures are resolved per member)
    for (const PassDesc& pd : p->plan.passes)
        for (int bi = pd.first_block; bi < pd.first_block + pd.nblocks; ++bi) {
            const BlockDesc& blk = p->plan.blocks[bi];
            for (int o = blk.first; !blk.generic && o < blk.first + blk.nops; ++o) {
                const int c = p->plan.ops[pd.first_op + o].tmpl;
                if (!((c >= 0 && c < kT_CODES) || (c >= kT_MIX1 && c < kT_MIX2 + 16))) {
                    delete p;
                    return fail(LSG_E_ARG, "internal planning error: operator code %d", c);
                }
            }
        }
    const int64_t base_entries = pool_entries;  // the caller's pool, then the relocated data
    pool_entries = base_entries + (int64_t)ext.size() / 2;
    size_t max_meta = 0;
    for (const PassDesc& pd : p->plan.passes)
        max_meta = std::max(max_meta, (size_t)pd.nops * (sizeof(TileOp) + 16) + (size_t)pd.nblocks * sizeof(BlockDesc));
    const size_t elt = lsg_elem_bytes(precision);
    p->smem = (elt << p->K) + max_meta;
    if (p->smem > 220 * 1024) {
        delete p;
        return fail(LSG_E_ARG, "a pass needs more than 220 KB of shared memory");
    }
    const size_t head0 = p->plan.passes.size() * sizeof(PassDesc) + p->plan.ops.size() * sizeof(TileOp) +
                         p->plan.blocks.size() * sizeof(BlockDesc);
    p->basis_off = (head0 + 15) & ~size_t(15);
    p->basis_passes = basis_passes(p->plan, nbits, precision, 0);
    p->basis_index = 0;
    const size_t head = p->basis_off + p->basis_passes.size() * sizeof(PassDesc);
    p->head_aligned = (head + 255) & ~size_t(255);
    const size_t total = p->head_aligned + (size_t)pool_entries * elt;
    std::vector<unsigned char> blob(std::max<size_t>(total, 1));
    std::memcpy(blob.data(), p->plan.passes.data(), p->plan.passes.size() * sizeof(PassDesc));
    std::memcpy(blob.data() + p->plan.passes.size() * sizeof(PassDesc), p->plan.ops.data(),
                p->plan.ops.size() * sizeof(TileOp));
    std::memcpy(blob.data() + p->plan.passes.size() * sizeof(PassDesc) + p->plan.ops.size() * sizeof(TileOp),
                p->plan.blocks.data(), p->plan.blocks.size() * sizeof(BlockDesc));
    std::memcpy(blob.data() + p->basis_off, p->basis_passes.data(), p->basis_passes.size() * sizeof(PassDesc));
    // the pool in the register precision: complex128 as is, complex64 rounded once, real
    // registers take the real parts (the imaginary ones are zero)
    auto put = [&](const double* src, int64_t n, unsigned char* dst) {
        if (precision == LSG_C128) {
            if (n) std::memcpy(dst, src, (size_t)n * 16);
        } else if (precision == LSG_C64) {
            float* f = reinterpret_cast<float*>(dst);
            for (int64_t i = 0; i < 2 * n; ++i) f[i] = (float)src[i];
        } else if (precision == LSG_R64) {
            double* d = reinterpret_cast<double*>(dst);
            for (int64_t i = 0; i < n; ++i) d[i] = src[2 * i];
        } else if (precision == LSG_RD) {  // each coefficient split into hi + lo
            DF* d = reinterpret_cast<DF*>(dst);
            for (int64_t i = 0; i < n; ++i) d[i] = DF(src[2 * i]);
        } else {
            float* f = reinterpret_cast<float*>(dst);
            for (int64_t i = 0; i < n; ++i) f[i] = (float)src[2 * i];
        }
    };
    unsigned char* dst = blob.data() + p->head_aligned;
    put(pool, base_entries, dst);
    put(ext.data(), (int64_t)ext.size() / 2, dst + (size_t)base_entries * elt);
    if (!upload) {
        p->pool_bytes.assign(dst, dst + (size_t)pool_entries * elt);
        *out = p;
        return LSG_OK;
    }
    int rc = ensure(p->dev, total);
    if (rc == LSG_OK) {
        // the host blob is released on return: the copy must have consumed it
        cudaError_t e = stream ? cudaMemcpyAsync(p->dev.ptr, blob.data(), total, cudaMemcpyHostToDevice, stream)
                               : cudaMemcpy(p->dev.ptr, blob.data(), total, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && stream) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) rc = fail(LSG_E_CUDA, "uploading the program failed: %s", cudaGetErrorString(e));
    }
    if (rc != LSG_OK) {
        release(p->dev);
        delete p;
        return rc;
    }
    *out = p;
    return LSG_OK;
}

int program_create_ex(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops, const double* pool,
                      int64_t pool_entries, const int* pred, const int* draw, const int* count, lsg_program_s** out,
                      cudaStream_t stream) {
    return program_build(nbits, precision, batch, ops, nops, pool, pool_entries, pred, draw, count, out, stream, true);
}

// Launch bound of specialized passes: CTAs per SM (the interpreter's pipe_ctas for the element).
static int jit_ctas(int precision) {
    if (t_choice.ctas) return std::max(1, std::min(4, t_choice.ctas));
    if (const char* env = getenv("LSG_JIT_CTAS")) return std::max(1, std::min(4, atoi(env)));
    // FP64 elements: one CTA (FP64-bound); double-float and complex64: two; real32: three
    return (precision == LSG_C128 || precision == LSG_R64) ? 1 : lsg_elem_bytes(precision) == 4 ? 3 : 2;
}

static int program_create(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops,
                          const double* pool, int64_t pool_entries, lsg_program_s** out, cudaStream_t stream) {
    LSG_CHECK(validate_ops(nbits, precision, batch, ops, nops, pool, pool_entries));
    return program_create_ex(nbits, precision, batch, ops, nops, pool, pool_entries, nullptr, nullptr, nullptr, out,
                             stream);
}

// A program for repeated runs (lsg_program_create): planned, uploaded, and its passes
// specialized at run time when they can be (the compiled module is cached by its source, so
// programs of the same shape share it).
static int program_create_jit(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops,
                              const double* pool, int64_t pool_entries, lsg_program_s** out, cudaStream_t stream) {
    LSG_CHECK(program_create(nbits, precision, batch, ops, nops, pool, pool_entries, out, stream));
    lsg_program_s* p = *out;
    const size_t eb = lsg_elem_bytes(precision);
    bool bulk = true;
    for (const PassDesc& pd : p->plan.passes) bulk = bulk && ((eb << pd.L) % 16) == 0;
    const int ctas = jit_ctas(precision);
    const int64_t bytes_per_run = 2 * ((int64_t)eb << nbits) * batch * (int64_t)p->plan.passes.size();
    const bool swz = jit_swizzle_fits(p->plan, eb, ((int64_t)eb << nbits) * batch);
    if (bulk && jit_wanted(bytes_per_run)) p->jit = jit_build(p->plan, precision, ctas, swz, jit_packed(precision));
    if (const char* path = getenv("LSG_JIT_DUMP")) {  // diagnostics: the specialized source of this program
        if (FILE* f = std::fopen(path, "w")) {
            const std::string src = jit_source(p->plan, precision, ctas, swz, jit_packed(precision));
            std::fwrite(src.data(), 1, src.size(), f);
            std::fclose(f);
        }
    }
    return LSG_OK;
}

void program_destroy(lsg_program_s* p) {
    if (!p) return;
    for (cudaEvent_t e : p->events) cudaEventDestroy(e);
    if (p->graph) cudaGraphExecDestroy(p->graph);
    release(p->dev);
    delete p;
}

static int program_launch(lsg_program_s* p, lsg_state_s* s, cudaEvent_t* marks, const TrajCtx& ctx, bool from_basis) {
    if (s->nbits != p->nbits || s->precision != p->precision || s->batch != p->batch)
        return fail(LSG_E_STATE, "the program was built for a register of %d bits, precision %d, batch %lld",
                    p->nbits, p->precision, (long long)p->batch);
    if (p->plan.passes.empty()) return LSG_OK;
    switch (s->precision) {
        case LSG_C128: return launch_passes<Cx<double>>(p, s, marks, ctx, from_basis);
        case LSG_C64: return launch_passes<Cx<float>>(p, s, marks, ctx, from_basis);
        case LSG_R64: return launch_passes<double>(p, s, marks, ctx, from_basis);
        case LSG_RD: return launch_passes<DF>(p, s, marks, ctx, from_basis);
        default: return launch_passes<float>(p, s, marks, ctx, from_basis);
    }
}

int program_run_ctx(lsg_program_s* p, lsg_state_s* s, cudaEvent_t* marks, const TrajCtx& ctx) {
    return program_launch(p, s, marks, ctx, false);
}

int set_basis_async(lsg_state_s* s, int64_t index);

// Make the program's device basis passes those of `index` (a complex register's fixed bits are the
// index's bits; a real register's do not depend on it), on the register's stream.
static int basis_passes_for(lsg_program_s* p, lsg_state_s* s, int64_t index) {
    if (s->real() || index == p->basis_index) return LSG_OK;
    p->basis_passes = basis_passes(p->plan, p->nbits, p->precision, index);
    void* dst = static_cast<unsigned char*>(p->dev.ptr) + p->basis_off;
    // pageable source: the copy is staged before the call returns
    LSG_CUDA(cudaMemcpyAsync(dst, p->basis_passes.data(), p->basis_passes.size() * sizeof(PassDesc),
                             cudaMemcpyHostToDevice, s->stream));
    p->basis_index = index;
    return LSG_OK;
}

// Set every member to basis state `index` and make the program's basis passes those of `index`
// (on the register's stream).
static int basis_prepare(lsg_program_s* p, lsg_state_s* s, int64_t index) {
    if (s->nbits != p->nbits || s->precision != p->precision || s->batch != p->batch)
        return fail(LSG_E_STATE, "the program was built for a register of %d bits, precision %d, batch %lld",
                    p->nbits, p->precision, (long long)p->batch);
    LSG_CHECK(set_basis_async(s, index));  // stream-ordered: no host wait before the passes
    return basis_passes_for(p, s, index);
}

// Set every member to basis state `index`, then run the passes on the tiles that can be nonzero.
static int program_run_basis(lsg_program_s* p, lsg_state_s* s, int64_t index, cudaEvent_t* marks) {
    LSG_CHECK(basis_prepare(p, s, index));
    return program_launch(p, s, marks, TrajCtx{}, true);
}

// Whether the pipelined interpreter takes this program's passes (bulk copies of its chunks, two
// tiles and the operators in shared memory).
template <typename T>
static bool pipe_eligible(const lsg_program_s* p) {
    const size_t tile_bytes = sizeof(T) << p->K;
    const int L = p->plan.passes.empty() ? 0 : p->plan.passes[0].L;
    return ((sizeof(T) << L) % 16) == 0 && getenv("LSG_NO_PIPELINE") == nullptr &&
           2 * tile_bytes + (p->smem - tile_bytes) <= 200 * 1024;
}

// Ragged run: launch k carries pass k (from a basis state) of every job that has one. Each job
// gets a range of the launch's CTAs in proportion to its tiles (at least one); the launch's
// shared memory is the largest any of its jobs needs. `ms`, when given, receives each launch's
// device time (events on `st`).
template <typename T>
static int launch_ragged(const std::vector<std::pair<lsg_program_s*, lsg_state_s*>>& jobs, cudaStream_t st,
                         float* ms) {
    size_t steps = 0;
    for (const auto& j : jobs) steps = std::max(steps, j.first->plan.passes.size());
    if (steps == 0) return LSG_OK;
    int dev = 0, sms = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    LSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int* status = device_status();
    if (!status) return fail(LSG_E_CUDA, "cannot allocate the device status word");
    const void* kern = PassKernels<T>::ragged();
    LSG_CHECK(allow_smem(kern));
    std::vector<RaggedJob> table;
    std::vector<size_t> first(steps), count(steps), smem(steps);
    std::vector<unsigned> grid(steps);
    for (size_t k = 0; k < steps; ++k) {
        first[k] = table.size();
        int64_t sum = 0;
        size_t need = 0;
        for (const auto& j : jobs) {
            const lsg_program_s* p = j.first;
            if (p->plan.passes.size() <= k) continue;
            const PassDesc& pd = p->basis_passes[k];
            const size_t tile_bytes = sizeof(T) << p->K;
            need = std::max(need, 2 * tile_bytes + (size_t)pd.nops * (sizeof(TileOp) + 16) +
                                      (size_t)pd.nblocks * sizeof(BlockDesc));
            sum += (1ll << pd.nouter) * p->batch;
        }
        int per_sm = 0;
        LSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPipeThreads, need));
        const double budget = (double)sms * std::max(per_sm, 1);
        int cta = 0;
        for (const auto& j : jobs) {
            lsg_program_s* p = j.first;
            lsg_state_s* s = j.second;
            if (p->plan.passes.size() <= k) continue;
            const PassDesc& pd = p->basis_passes[k];
            RaggedJob r;
            r.state = s->data;
            r.member_elems = s->elems;
            const PassDesc* plan_pd_dev = reinterpret_cast<const PassDesc*>(p->dev.ptr);
            r.ops = reinterpret_cast<const TileOp*>(plan_pd_dev + p->plan.passes.size());
            r.blocks = reinterpret_cast<const BlockDesc*>(r.ops + p->plan.ops.size());
            r.pass = reinterpret_cast<const PassDesc*>(static_cast<unsigned char*>(p->dev.ptr) + p->basis_off) + k;
            r.data = static_cast<unsigned char*>(p->dev.ptr) + p->head_aligned;
            r.tiles_per_member = 1ll << pd.nouter;
            r.total_tiles = r.tiles_per_member * p->batch;
            const int64_t want = (int64_t)std::llround(budget * (double)r.total_tiles / (double)sum);
            r.ctas = (int)std::max<int64_t>(1, std::min<int64_t>(want, r.total_tiles));
            r.cta0 = cta;
            cta += r.ctas;
            table.push_back(r);
        }
        count[k] = table.size() - first[k];
        smem[k] = need;
        grid[k] = (unsigned)cta;
    }
    RaggedJob* dtab = nullptr;
    LSG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dtab), table.size() * sizeof(RaggedJob), st));
    // pageable source: staged before the call returns
    LSG_CUDA(cudaMemcpyAsync(dtab, table.data(), table.size() * sizeof(RaggedJob), cudaMemcpyHostToDevice, st));
    std::vector<cudaEvent_t> marks;
    if (ms) {
        marks.resize(steps + 1);
        for (auto& e : marks) LSG_CUDA(cudaEventCreate(&e));
    }
    for (size_t k = 0; k < steps; ++k) {
        if (ms) LSG_CUDA(cudaEventRecord(marks[k], st));
        PassKernels<T>::launch_ragged(grid[k], smem[k], st, dtab + first[k], (int)count[k], status);
    }
    if (ms) LSG_CUDA(cudaEventRecord(marks[steps], st));
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaFreeAsync(dtab, st));
    if (ms) {
        LSG_CUDA(cudaEventSynchronize(marks[steps]));
        for (size_t k = 0; k < steps; ++k) LSG_CUDA(cudaEventElapsedTime(&ms[k], marks[k], marks[k + 1]));
        for (auto& e : marks) cudaEventDestroy(e);
    }
    return LSG_OK;
}

static int program_run(lsg_program_s* p, lsg_state_s* s, cudaEvent_t* marks) {
    return program_run_ctx(p, s, marks, TrajCtx{});
}

int apply_ops(lsg_state_s* s, const lsg_op* ops, int32_t nops, const double* pool, int64_t pool_entries) {
    if (nops == 0) return validate_ops(s->nbits, s->precision, s->batch, ops, nops, pool, pool_entries);
    lsg_program_s* p = nullptr;
    LSG_CHECK(program_create(s->nbits, s->precision, s->batch, ops, nops, pool, pool_entries, &p, s->stream));
    int rc = program_run(p, s, nullptr);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    program_destroy(p);
    LSG_CHECK(rc);
    if (e != cudaSuccess) return fail(LSG_E_CUDA, "the passes failed: %s", cudaGetErrorString(e));
    return check_device_status(s->stream);
}

// Set every member to basis state `index` and apply `ops` from it, skipping tiles that are still
// zero (program_run_basis); the result equals set_basis + apply_ops.
int apply_ops_basis(lsg_state_s* s, int64_t index, const lsg_op* ops, int32_t nops, const double* pool,
                    int64_t pool_entries) {
    if (nops == 0) {
        LSG_CHECK(validate_ops(s->nbits, s->precision, s->batch, ops, nops, pool, pool_entries));
        LSG_CHECK(set_basis_async(s, index));
        LSG_CUDA(cudaStreamSynchronize(s->stream));
        return LSG_OK;
    }
    lsg_program_s* p = nullptr;
    LSG_CHECK(program_create(s->nbits, s->precision, s->batch, ops, nops, pool, pool_entries, &p, s->stream));
    int rc = program_run_basis(p, s, index, nullptr);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    program_destroy(p);
    LSG_CHECK(rc);
    if (e != cudaSuccess) return fail(LSG_E_CUDA, "the passes failed: %s", cudaGetErrorString(e));
    return check_device_status(s->stream);
}

// ------------------------------------------------------------------------ register kernels

// After a zero fill: member m's element `index` of a complex register set to 1.
template <typename R>
__global__ void k_basis_one(Cx<R>* state, int64_t elems, int64_t batch, int64_t index) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < batch; m += (int64_t)gridDim.x * blockDim.x)
        state[m * elems + index] = Cx<R>(R(1), R(0));
}

// After a zero fill: the Pauli-transfer form of |b><b| on n qubits, r_P = <b|P|b>, which is
// (-1)^{|z & b|} for the 2^n diagonal Paulis (x = 0: register index z below 2^n) of every member
// (the others stay 0).
template <typename R>
__global__ void k_basis_diag_ptm(R* state, int64_t elems, int64_t batch, int n, int64_t b) {
    const int64_t zmax = 1ll << n, total = zmax * batch;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i >> n, z = i & (zmax - 1);
        state[m * elems + z] = (__popcll((unsigned long long)(z & b)) & 1) ? R(-1) : R(1);
    }
}

template <typename R, typename C>
__global__ void k_real_to_complex(const R* in, Cx<C>* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = Cx<C>((C)(double)in[i], C(0));
}

__global__ void k_r32_to_r64(const float* in, double* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

__global__ void k_r64_to_r32(const double* in, float* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void k_r64_to_rd(const double* in, DF* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = DF(in[i]);
}

__global__ void k_rd_to_r64(const DF* in, double* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

__global__ void k_c128_to_c64(const double2* in, float2* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

__global__ void k_c64_to_c128(const float2* in, double2* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

unsigned grid_for(int64_t n, int threads = 256) {
    int64_t g = (n + threads - 1) / threads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

// Every member to basis state `index`, enqueued on the register's stream: a zero fill at the
// copy engine's write rate, then the nonzero entries.
int set_basis_async(lsg_state_s* s, int64_t index) {
    const int64_t limit = s->real() ? (1ll << (s->nbits / 2)) : s->elems;  // real: |index><index| of nbits/2 qubits
    if (index < 0 || index >= limit) return fail(LSG_E_ARG, "basis index %lld out of range", (long long)index);
    LSG_CUDA(cudaMemsetAsync(s->data, 0, s->member_bytes() * (size_t)s->batch, s->stream));
    const int n = s->nbits / 2;
    if (s->precision == LSG_C128)
        k_basis_one<double><<<grid_for(s->batch), 256, 0, s->stream>>>((Cx<double>*)s->data, s->elems, s->batch, index);
    else if (s->precision == LSG_C64)
        k_basis_one<float><<<grid_for(s->batch), 256, 0, s->stream>>>((Cx<float>*)s->data, s->elems, s->batch, index);
    else if (s->precision == LSG_R64)
        k_basis_diag_ptm<double><<<grid_for(s->batch << n), 256, 0, s->stream>>>((double*)s->data, s->elems, s->batch, n, index);
    else if (s->precision == LSG_RD)
        k_basis_diag_ptm<DF><<<grid_for(s->batch << n), 256, 0, s->stream>>>((DF*)s->data, s->elems, s->batch, n, index);
    else
        k_basis_diag_ptm<float><<<grid_for(s->batch << n), 256, 0, s->stream>>>((float*)s->data, s->elems, s->batch, n, index);
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

}  // namespace lsg

using namespace lsg;

extern "C" {

const char* lsg_last_error(void) { return lsg::t_error.c_str(); }

int lsg_version(void) { return 1; }

int lsg_init(int device) {
    clear_error();
    int count = 0;
    LSG_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return fail(LSG_E_ARG, "device %d does not exist (%d visible)", device, count);
    LSG_CUDA(cudaSetDevice(device));
    cudaMemPool_t mp;
    if (cudaDeviceGetDefaultMemPool(&mp, device) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return LSG_OK;
}

int lsg_max_bits(void) { return kMaxBits; }

int lsg_mem_info(int64_t* free_bytes, int64_t* total_bytes) {
    clear_error();
    size_t f = 0, t = 0;
    LSG_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (int64_t)f;
    if (total_bytes) *total_bytes = (int64_t)t;
    return LSG_OK;
}

int lsg_state_create(int nbits, int precision, int64_t batch, lsg_state* out) {
    clear_error();
    if (!out) return fail(LSG_E_ARG, "lsg_state_create: null output");
    *out = nullptr;
    if (nbits < 0) return fail(LSG_E_ARG, "lsg_state_create: negative bit count");
    if (nbits > kMaxBits) return fail(LSG_E_CAPACITY, "a register of %d bits exceeds the engine's %d", nbits, kMaxBits);
    if (precision < LSG_C128 || precision > LSG_RD) return fail(LSG_E_ARG, "unknown precision %d", precision);
    if ((lsg_precision_real(precision)) && (nbits & 1))
        return fail(LSG_E_ARG, "a Pauli-transfer register has an even number of bits (two per qubit)");
    if (batch < 1) return fail(LSG_E_ARG, "lsg_state_create: batch must be at least 1");
    static std::atomic<uint64_t> next_uid{0};
    auto* s = new lsg_state_s();
    s->nbits = nbits;
    s->precision = precision;
    s->batch = batch;
    s->elems = 1ll << nbits;
    s->uid = ++next_uid;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail(LSG_E_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(e));
    }
    s->program.stream = s->scratch.stream = s->scratch2.stream = s->stream;
    e = cudaMallocAsync(&s->data, s->member_bytes() * (size_t)batch, s->stream);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s->stream);
        delete s;
        cudaGetLastError();
        return fail(LSG_E_MEMORY, "cannot allocate %lld bytes of device memory for the register",
                    (long long)(s->member_bytes() * (size_t)batch));
    }
    *out = s;
    return set_basis_async(s, 0);  // stream-ordered like all work on the register: no host wait
}

int lsg_state_free(lsg_state s) {
    clear_error();
    if (!s) return LSG_OK;
    cudaFreeAsync(s->data, s->stream);
    release(s->program);
    release(s->scratch);
    release(s->scratch2);
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
    delete s;
    return LSG_OK;
}

int lsg_state_set_basis(lsg_state s, int64_t index) {
    clear_error();
    if (!s) return fail(LSG_E_ARG, "null register");
    LSG_CHECK(set_basis_async(s, index));
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_state_upload(lsg_state s, const double* host, int64_t nbytes) {
    clear_error();
    if (!s || !host) return fail(LSG_E_ARG, "null argument");
    const int64_t n = s->elems * s->batch;
    const int64_t want = n * (s->real() ? 8 : 16);  // float64 per element for real registers
    if (nbytes != want) return fail(LSG_E_ARG, "upload expects %lld bytes, got %lld", (long long)want, (long long)nbytes);
    if (s->precision == LSG_C128 || s->precision == LSG_R64) {
        LSG_CUDA(cudaMemcpyAsync(s->data, host, (size_t)nbytes, cudaMemcpyHostToDevice, s->stream));
    } else {
        LSG_CHECK(ensure(s->scratch2, (size_t)nbytes));
        LSG_CUDA(cudaMemcpyAsync(s->scratch2.ptr, host, (size_t)nbytes, cudaMemcpyHostToDevice, s->stream));
        if (s->precision == LSG_R32)
            k_r64_to_r32<<<grid_for(n), 256, 0, s->stream>>>((const double*)s->scratch2.ptr, (float*)s->data, n);
        else if (s->precision == LSG_RD)
            k_r64_to_rd<<<grid_for(n), 256, 0, s->stream>>>((const double*)s->scratch2.ptr, (DF*)s->data, n);
        else
            k_c128_to_c64<<<grid_for(n), 256, 0, s->stream>>>((const double2*)s->scratch2.ptr, (float2*)s->data, n);
        LSG_CUDA(cudaGetLastError());
    }
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_state_download(lsg_state s, double* host, int64_t nbytes) {
    clear_error();
    if (!s || !host) return fail(LSG_E_ARG, "null argument");
    const int64_t n = s->elems * s->batch;
    const int64_t want = n * (s->real() ? 8 : 16);
    if (nbytes != want) return fail(LSG_E_ARG, "download expects %lld bytes, got %lld", (long long)want, (long long)nbytes);
    if (s->precision == LSG_C128 || s->precision == LSG_R64) {
        LSG_CUDA(cudaMemcpyAsync(host, s->data, (size_t)nbytes, cudaMemcpyDeviceToHost, s->stream));
    } else {
        LSG_CHECK(ensure(s->scratch2, (size_t)nbytes));
        if (s->precision == LSG_R32)
            k_r32_to_r64<<<grid_for(n), 256, 0, s->stream>>>((const float*)s->data, (double*)s->scratch2.ptr, n);
        else if (s->precision == LSG_RD)
            k_rd_to_r64<<<grid_for(n), 256, 0, s->stream>>>((const DF*)s->data, (double*)s->scratch2.ptr, n);
        else
            k_c64_to_c128<<<grid_for(n), 256, 0, s->stream>>>((const float2*)s->data, (double2*)s->scratch2.ptr, n);
        LSG_CUDA(cudaGetLastError());
        LSG_CUDA(cudaMemcpyAsync(host, s->scratch2.ptr, (size_t)nbytes, cudaMemcpyDeviceToHost, s->stream));
    }
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_state_bytes(lsg_state s, int64_t* out) {
    clear_error();
    if (!s || !out) return fail(LSG_E_ARG, "null argument");
    *out = (int64_t)(s->member_bytes() * (size_t)s->batch + s->program.bytes + s->scratch.bytes + s->scratch2.bytes);
    return LSG_OK;
}

int lsg_apply(lsg_state s, const lsg_op* ops, int32_t nops, const double* pool, int64_t pool_entries) {
    clear_error();
    if (!s) return fail(LSG_E_ARG, "null register");
    return apply_ops(s, ops, nops, pool, pool_entries);
}

int lsg_apply_from_basis(lsg_state s, int64_t index, const lsg_op* ops, int32_t nops, const double* pool,
                         int64_t pool_entries) {
    clear_error();
    if (!s) return fail(LSG_E_ARG, "null register");
    return apply_ops_basis(s, index, ops, nops, pool, pool_entries);
}


int lsg_state_sync(lsg_state s) {
    clear_error();
    if (!s) return fail(LSG_E_ARG, "null register");
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return check_device_status(s->stream);
}

int lsg_state_stream(lsg_state s, void** stream) {
    clear_error();
    if (!s || !stream) return fail(LSG_E_ARG, "null argument");
    *stream = (void*)s->stream;
    return LSG_OK;
}

int lsg_state_to_complex(lsg_state src, int64_t member, lsg_state dst) {
    clear_error();
    if (!src || !dst) return fail(LSG_E_ARG, "null register");
    if (!src->real() || dst->real()) return fail(LSG_E_ARG, "lsg_state_to_complex: from a real register to a complex one");
    if (src->nbits != dst->nbits) return fail(LSG_E_ARG, "lsg_state_to_complex: registers of different sizes");
    if (member < 0 || member >= src->batch) return fail(LSG_E_ARG, "member %lld out of range", (long long)member);
    LSG_CUDA(cudaStreamSynchronize(src->stream));  // dst's stream reads what src's stream wrote
    const int64_t n = src->elems;
    const unsigned g = grid_for(n);
    if (src->precision == LSG_RD && dst->precision == LSG_C128)
        k_real_to_complex<DF, double><<<g, 256, 0, dst->stream>>>((const DF*)src->data + member * n, (Cx<double>*)dst->data, n);
    else if (src->precision == LSG_RD)
        k_real_to_complex<DF, float><<<g, 256, 0, dst->stream>>>((const DF*)src->data + member * n, (Cx<float>*)dst->data, n);
    else if (src->precision == LSG_R64 && dst->precision == LSG_C128)
        k_real_to_complex<double, double><<<g, 256, 0, dst->stream>>>((const double*)src->data + member * n, (Cx<double>*)dst->data, n);
    else if (src->precision == LSG_R64)
        k_real_to_complex<double, float><<<g, 256, 0, dst->stream>>>((const double*)src->data + member * n, (Cx<float>*)dst->data, n);
    else if (dst->precision == LSG_C128)
        k_real_to_complex<float, double><<<g, 256, 0, dst->stream>>>((const float*)src->data + member * n, (Cx<double>*)dst->data, n);
    else
        k_real_to_complex<float, float><<<g, 256, 0, dst->stream>>>((const float*)src->data + member * n, (Cx<float>*)dst->data, n);
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaStreamSynchronize(dst->stream));
    return LSG_OK;
}

int lsg_program_create(lsg_state shape, const lsg_op* ops, int32_t nops, const double* pool, int64_t pool_entries,
                       lsg_program* out) {
    clear_error();
    if (!shape || !out) return fail(LSG_E_ARG, "null argument");
    *out = nullptr;
    LSG_CHECK(program_create_jit(shape->nbits, shape->precision, shape->batch, ops, nops, pool, pool_entries, out,
                                 shape->stream));
    // The program outlives no stream of `shape`: the register may be freed first (its stream
    // destroyed), so the program's memory is released with cudaFree, which waits for the device.
    (*out)->dev.stream = nullptr;
    return LSG_OK;
}

int lsg_program_create_opts(lsg_state shape, const lsg_op* ops, int32_t nops, const double* pool,
                            int64_t pool_entries, const lsg_plan_opts* opts, lsg_program* out) {
    clear_error();
    if (!shape || !out) return fail(LSG_E_ARG, "null argument");
    *out = nullptr;
    PlanChoice c;
    if (opts) {
        const int eb_log = lsg_elem_bytes(shape->precision) == 16 ? 4 : lsg_elem_bytes(shape->precision) == 8 ? 3 : 2;
        // a tile of at most 64 KB (two of them and the pass metadata fit shared memory); runs of at
        // least 16 bytes (bulk copies); 1 to 4 CTAs per SM; 1 to 192 operators per pass
        if (opts->tile_bits < 0 || (opts->tile_bits && opts->tile_bits + eb_log > 16))
            return fail(LSG_E_ARG, "lsg_program_create_opts: tile of 2^%d elements exceeds 64 KB", opts->tile_bits);
        if (opts->low_bits < 0 || (opts->low_bits && opts->low_bits + eb_log < 4))
            return fail(LSG_E_ARG, "lsg_program_create_opts: runs of 2^%d elements are under 16 bytes", opts->low_bits);
        if (opts->tile_bits && opts->low_bits && opts->low_bits > opts->tile_bits)
            return fail(LSG_E_ARG, "lsg_program_create_opts: more low bits than tile bits");
        if (opts->ctas < 0 || opts->ctas > 4) return fail(LSG_E_ARG, "lsg_program_create_opts: 1 to 4 CTAs per SM");
        if (opts->max_ops < 0 || opts->max_ops > kMaxPassOps)
            return fail(LSG_E_ARG, "lsg_program_create_opts: 1 to %d operators per pass", kMaxPassOps);
        c = PlanChoice{opts->tile_bits, opts->low_bits, opts->ctas, opts->max_ops};
    }
    struct Restore {
        PlanChoice saved = t_choice;
        ~Restore() { t_choice = saved; }
    } restore;
    t_choice = c;
    LSG_CHECK(program_create_jit(shape->nbits, shape->precision, shape->batch, ops, nops, pool, pool_entries, out,
                                 shape->stream));
    (*out)->dev.stream = nullptr;  // as lsg_program_create: the program may outlive the register
    return LSG_OK;
}

int lsg_program_run(lsg_program p, lsg_state s) {
    clear_error();
    if (!p || !s) return fail(LSG_E_ARG, "null argument");
    return program_run(p, s, nullptr);
}

int lsg_program_run_timed(lsg_program p, lsg_state s, float* pass_ms) {
    clear_error();
    if (!p || !s || !pass_ms) return fail(LSG_E_ARG, "null argument");
    const size_t need = p->plan.passes.size() + 1;
    while (p->events.size() < need) {
        cudaEvent_t e;
        LSG_CUDA(cudaEventCreate(&e));
        p->events.push_back(e);
    }
    LSG_CHECK(program_run(p, s, p->events.data()));
    LSG_CUDA(cudaEventSynchronize(p->events[need - 1]));
    for (size_t i = 0; i + 1 < need; ++i) LSG_CUDA(cudaEventElapsedTime(&pass_ms[i], p->events[i], p->events[i + 1]));
    return check_device_status(s->stream);
}

int lsg_program_run_from_basis(lsg_program p, lsg_state s, int64_t index, float* pass_ms) {
    clear_error();
    if (!p || !s) return fail(LSG_E_ARG, "null argument");
    if (!pass_ms) return program_run_basis(p, s, index, nullptr);
    const size_t need = p->plan.passes.size() + 1;
    while (p->events.size() < need) {
        cudaEvent_t e;
        LSG_CUDA(cudaEventCreate(&e));
        p->events.push_back(e);
    }
    LSG_CHECK(program_run_basis(p, s, index, p->events.data()));
    LSG_CUDA(cudaEventSynchronize(p->events[need - 1]));
    for (size_t i = 0; i + 1 < need; ++i) LSG_CUDA(cudaEventElapsedTime(&pass_ms[i], p->events[i], p->events[i + 1]));
    return check_device_status(s->stream);
}

int lsg_programs_run_ragged(int32_t count, const lsg_program* programs, const lsg_state* states, const int64_t* index,
                           float* step_ms) {
    clear_error();
    if (count < 1 || !programs || !states) return fail(LSG_E_ARG, "lsg_programs_run_ragged: bad arguments");
    const int precision = states[0] ? states[0]->precision : -1;
    for (int32_t i = 0; i < count; ++i) {
        if (!programs[i] || !states[i]) return fail(LSG_E_ARG, "lsg_programs_run_ragged: null program or register %d", i);
        if (states[i]->precision != precision)
            return fail(LSG_E_ARG, "lsg_programs_run_ragged: register %d has another precision than register 0", i);
        for (int32_t j = 0; j < i; ++j) {
            if (states[j] == states[i]) return fail(LSG_E_ARG, "lsg_programs_run_ragged: register %d appears twice", i);
            // one program's basis passes live in its device memory: shared only by equal indices
            if (programs[j] == programs[i] && !states[i]->real() && (index ? index[i] != index[j] : false))
                return fail(LSG_E_ARG, "lsg_programs_run_ragged: program %d appears again with another basis index", i);
        }
    }
    cudaStream_t st = states[0]->stream;
    std::vector<std::pair<lsg_program_s*, lsg_state_s*>> ragged;
    std::vector<cudaEvent_t> events;
    auto cleanup = [&]() {
        for (cudaEvent_t e : events) cudaEventDestroy(e);
    };
    int rc = LSG_OK;
    for (int32_t i = 0; i < count && rc == LSG_OK; ++i) {
        lsg_program_s* p = programs[i];
        lsg_state_s* s = states[i];
        rc = basis_prepare(p, s, index ? index[i] : 0);
        if (rc != LSG_OK) break;
        bool eligible;
        switch (precision) {
            case LSG_C128: eligible = pipe_eligible<Cx<double>>(p); break;
            case LSG_C64: eligible = pipe_eligible<Cx<float>>(p); break;
            case LSG_R64: eligible = pipe_eligible<double>(p); break;
            case LSG_RD: eligible = pipe_eligible<DF>(p); break;
            default: eligible = pipe_eligible<float>(p); break;
        }
        if (!eligible) {  // this one runs alone on its own stream
            rc = program_launch(p, s, nullptr, TrajCtx{}, true);
            continue;
        }
        if (p->plan.passes.empty()) continue;
        ragged.emplace_back(p, s);
        if (s->stream != st) {  // the ragged launches go after this register's basis state
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                rc = fail(LSG_E_CUDA, "lsg_programs_run_ragged: cannot create an event");
                break;
            }
            events.push_back(e);
            if (cudaEventRecord(e, s->stream) != cudaSuccess || cudaStreamWaitEvent(st, e, 0) != cudaSuccess)
                rc = fail(LSG_E_CUDA, "lsg_programs_run_ragged: cannot order the streams");
        }
    }
    if (rc == LSG_OK && !ragged.empty()) {
        switch (precision) {
            case LSG_C128: rc = launch_ragged<Cx<double>>(ragged, st, step_ms); break;
            case LSG_C64: rc = launch_ragged<Cx<float>>(ragged, st, step_ms); break;
            case LSG_R64: rc = launch_ragged<double>(ragged, st, step_ms); break;
            case LSG_RD: rc = launch_ragged<DF>(ragged, st, step_ms); break;
            default: rc = launch_ragged<float>(ragged, st, step_ms); break;
        }
    }
    if (rc == LSG_OK) {  // later work on every register goes after the ragged launches
        cudaEvent_t done;
        if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
            rc = fail(LSG_E_CUDA, "lsg_programs_run_ragged: cannot create an event");
        } else {
            events.push_back(done);
            if (cudaEventRecord(done, st) != cudaSuccess) rc = fail(LSG_E_CUDA, "lsg_programs_run_ragged: event record");
            for (const auto& j : ragged)
                if (rc == LSG_OK && j.second->stream != st && cudaStreamWaitEvent(j.second->stream, done, 0) != cudaSuccess)
                    rc = fail(LSG_E_CUDA, "lsg_programs_run_ragged: cannot order the streams");
        }
    }
    cleanup();  // events already recorded are released when they complete
    return rc;
}

int lsg_program_set_data(lsg_program p, lsg_state s, const lsg_op* ops, int32_t nops, const double* pool,
                         int64_t pool_entries) {
    clear_error();
    if (!p || !s) return fail(LSG_E_ARG, "null argument");
    if (s->nbits != p->nbits || s->precision != p->precision || s->batch != p->batch)
        return fail(LSG_E_STATE, "the program was built for a register of %d bits, precision %d, batch %lld",
                    p->nbits, p->precision, (long long)p->batch);
    LSG_CHECK(validate_ops(p->nbits, p->precision, p->batch, ops, nops, pool, pool_entries));
    // the same operator table (kinds, bits, data offsets): the program's plan holds for it
    if (p->src_ops.empty() || (size_t)nops != p->src_ops.size() ||
        std::memcmp(ops, p->src_ops.data(), (size_t)nops * sizeof(lsg_op)) != 0)
        return fail(LSG_E_STATE, "lsg_program_set_data: the operators plan differently from the program's (another "
                                 "structure): build a new program");
    lsg_program_s* q = nullptr;
    const PlanChoice keep = t_choice;  // the plan choices the program was made with
    t_choice = p->choice;
    const int rc = program_build(p->nbits, p->precision, p->batch, ops, nops, pool, pool_entries, nullptr, nullptr,
                                 nullptr, &q, nullptr, false, &p->raw_plan);
    t_choice = keep;
    LSG_CHECK(rc);
    auto same_bytes = [](const auto& a, const auto& b) {
        return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(a[0])) == 0);
    };
    const bool same = q->K == p->K && same_bytes(q->plan.passes, p->plan.passes) && same_bytes(q->plan.ops, p->plan.ops) &&
                      same_bytes(q->plan.blocks, p->plan.blocks) &&
                      p->head_aligned + q->pool_bytes.size() <= p->dev.bytes;
    if (!same) {
        program_destroy(q);
        return fail(LSG_E_STATE, "lsg_program_set_data: the operators plan differently from the program's (another "
                                 "structure): build a new program");
    }
    // after the register's earlier work (a run may still read the old data); pageable source:
    // staged before the call returns
    const cudaError_t e = cudaMemcpyAsync(static_cast<unsigned char*>(p->dev.ptr) + p->head_aligned, q->pool_bytes.data(),
                                          q->pool_bytes.size(), cudaMemcpyHostToDevice, s->stream);
    program_destroy(q);
    if (e != cudaSuccess) return fail(LSG_E_CUDA, "lsg_program_set_data: %s", cudaGetErrorString(e));
    return LSG_OK;
}

int lsg_program_graph_run(lsg_program p, lsg_state s, int64_t index) {
    clear_error();
    if (!p || !s) return fail(LSG_E_ARG, "null argument");
    if (!p->graph || p->graph_uid != s->uid || p->graph_index != index) {
        if (p->graph) {
            cudaGraphExecDestroy(p->graph);
            p->graph = nullptr;
        }
        // everything that is not a stream operation happens before the capture: the basis passes
        // for `index` (a host copy), the device status word, kernel attributes (a first run)
        LSG_CHECK(program_run_basis(p, s, index, nullptr));
        cudaGraph_t graph = nullptr;
        LSG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = set_basis_async(s, index);
        if (rc == LSG_OK) rc = program_launch(p, s, nullptr, TrajCtx{}, true);
        const cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (rc == LSG_OK && e != cudaSuccess) rc = fail(LSG_E_CUDA, "capturing the program: %s", cudaGetErrorString(e));
        if (rc == LSG_OK && cudaGraphInstantiate(&p->graph, graph, 0) != cudaSuccess) {
            p->graph = nullptr;
            rc = fail(LSG_E_CUDA, "instantiating the program's graph failed");
        }
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (rc != LSG_OK) return rc;
        p->graph_uid = s->uid;
        p->graph_index = index;
        return LSG_OK;  // this call's run was the plain one before the capture
    }
    LSG_CHECK(basis_passes_for(p, s, index));  // another index may have run in between
    LSG_CUDA(cudaGraphLaunch(p->graph, s->stream));
    return LSG_OK;
}

int lsg_program_basis_info(lsg_program p, int64_t* bytes_per_run, int64_t* tiles_per_run) {
    clear_error();
    if (!p) return fail(LSG_E_ARG, "null program");
    int64_t tiles = 0;
    for (const PassDesc& pd : p->basis_passes) tiles += (1ll << pd.nouter) * p->batch;
    if (tiles_per_run) *tiles_per_run = tiles;
    if (bytes_per_run) *bytes_per_run = 2 * tiles * ((int64_t)lsg_elem_bytes(p->precision) << p->K);
    return LSG_OK;
}

// Floating-point operations per register element that one operator of a pass executes (a
// multiply or add counts 1, a fused multiply-add 2), as the register-block functions and the
// shared-memory operators compute them.
static double op_flops_per_element(const lsg::TileOp& op, bool complex_elems) {
    using namespace lsg;
    const int c = op.tmpl;
    const double mul = complex_elems ? 6.0 : 1.0;  // one (complex) product per element
    if (c >= kT_DENSE1 && c < kT_DENSE1 + 4) return complex_elems ? 14.0 : 3.0;
    if (c >= kT_DENSE2 && c < kT_DENSE2 + 16) return complex_elems ? 30.0 : 7.0;
    if (c >= kT_TPD2 && c < kT_TPD2 + 16) {  // rows 1-3: a product, then a multiply-add per further term
        double f = 0.0;
        for (int r = 0; r < 3; ++r) {
            const int terms = 4 - __builtin_popcount((unsigned)(op.zmask >> (4 * r)) & 15u);
            f += terms ? 1.0 + 2.0 * (terms - 1) : 0.0;
        }
        return f / 4.0;
    }
    if ((c >= kT_PERM1 && c < kT_PERM1 + 4) || (c >= kT_PERM2 && c < kT_PERM2 + 16)) return mul;
    if (c == kT_DIAGB || c == kT_SCALE || c == kT_DIAG) return mul;
    if (c == kT_DENSEB) return (complex_elems ? 8.0 : 2.0) * (double)(1 << op.k);
    if ((c >= kT_DEPOL1 && c < kT_DEPOL1 + 16) || c == kT_DEPOL2) return 4.0;
    if ((c >= kT_X1 && c < kT_X1 + 4) || (c >= kT_CX && c < kT_CX + 16) || (c >= kT_SWAP && c < kT_SWAP + 16)) return 0.0;
    if ((c >= kT_MIX1 && c < kT_MIX1 + 4) || (c >= kT_MIX2 && c < kT_MIX2 + 16)) return complex_elems ? 30.0 : 7.0;
    // the shared-memory path: a dense 2^k operator is 2^k (complex) multiply-adds per element
    const double fma = complex_elems ? 8.0 : 2.0;
    switch (op.kind) {
        case LSG_OP_MATRIX: return fma * (double)(1 << op.k);
        case LSG_OP_DEPOL: return 4.0;
        default: return mul;
    }
}

int lsg_program_pass_info(lsg_program p, int32_t cap, int64_t* bytes, double* flops_per_element, int32_t* blocks) {
    clear_error();
    if (!p) return fail(LSG_E_ARG, "null program");
    const int32_t n = (int32_t)p->plan.passes.size();
    if (cap < n) return fail(LSG_E_ARG, "lsg_program_pass_info: room for %d passes, the program has %d", cap, n);
    const bool cx = !lsg_precision_real(p->precision);
    for (int32_t i = 0; i < n; ++i) {
        const lsg::PassDesc& pd = p->plan.passes[(size_t)i];
        const lsg::PassDesc& visited = p->basis_passes.size() == (size_t)n ? p->basis_passes[(size_t)i] : pd;
        if (bytes) bytes[i] = 2 * (1ll << visited.nouter) * p->batch * ((int64_t)lsg_elem_bytes(p->precision) << pd.K);
        if (blocks) blocks[i] = pd.nblocks;
        if (flops_per_element) {
            double f = 0.0;
            for (int k = 0; k < pd.nops; ++k) f += op_flops_per_element(p->plan.ops[(size_t)(pd.first_op + k)], cx);
            flops_per_element[i] = f;
        }
    }
    return LSG_OK;
}

int lsg_program_info(lsg_program p, int32_t* passes, int64_t* bytes_per_run) {
    clear_error();
    if (!p) return fail(LSG_E_ARG, "null program");
    const int64_t member = (int64_t)lsg_elem_bytes(p->precision) << p->nbits;
    if (passes) *passes = (int32_t)p->plan.passes.size();
    if (bytes_per_run) *bytes_per_run = 2 * member * p->batch * (int64_t)p->plan.passes.size();
    return LSG_OK;
}

int lsg_program_specialized(lsg_program p) {
    clear_error();
    if (!p) return fail(LSG_E_ARG, "null program");
    return p->jit ? 1 : 0;
}

int lsg_jit_wanted(int64_t bytes_per_run) {
    clear_error();
    if (bytes_per_run < 0) return fail(LSG_E_ARG, "negative byte count");
    return jit_wanted(bytes_per_run) ? 1 : 0;
}

int lsg_program_source(int nbits, int precision, int64_t batch, const lsg_op* ops, int32_t nops, const double* pool,
                       int64_t pool_entries, int compile, char* buf, int64_t cap, int64_t* len) {
    clear_error();
    if (nbits < 0 || nbits > kMaxBits || batch < 1) return fail(LSG_E_ARG, "bad register shape");
    LSG_CHECK(validate_ops(nbits, precision, batch, ops, nops, pool, pool_entries));
    lsg_program_s* p = nullptr;
    LSG_CHECK(program_build(nbits, precision, batch, ops, nops, pool, pool_entries, nullptr, nullptr, nullptr, &p,
                            nullptr, false));
    const size_t eb = lsg_elem_bytes(precision);
    const std::string src =
        jit_source(p->plan, precision, jit_ctas(precision), jit_swizzle_fits(p->plan, eb, ((int64_t)eb << nbits) * batch),
                   jit_packed(precision));
    delete p;
    if (len) *len = (int64_t)src.size();
    if (buf && cap > 0) {
        const size_t n = std::min<size_t>(src.size(), (size_t)cap - 1);
        std::memcpy(buf, src.data(), n);
        buf[n] = '\0';
    }
    if (compile && !src.empty()) return jit_compile_check(src);
    return LSG_OK;
}

int lsg_plan(int nbits, int precision, const lsg_op* ops, int32_t nops, int32_t* passes) {
    clear_error();
    if (!passes || nops < 0 || (nops > 0 && !ops)) return fail(LSG_E_ARG, "bad arguments");
    if (nbits < 0 || nbits > kMaxBits) return fail(LSG_E_CAPACITY, "a register of %d bits exceeds the engine's %d", nbits, kMaxBits);
    for (int i = 0; i < nops; ++i)
        if (!op_bits_ok(ops[i], nbits)) return fail(LSG_E_ARG, "operator %d has a bad kind or bits", i);
    const int K = tile_bits_for(nbits, precision);
    const int L = std::min(K, low_bits_for(nbits, precision));
    Plan plan = plan_passes(ops, nops, nbits, K, L, block_bits_for(precision));
    if (nops > 0 && plan.passes.empty()) return fail(LSG_E_ARG, "an operator does not fit a tile of %d bits", K);
    LSG_CHECK(check_plan(plan));
    *passes = (int32_t)plan.passes.size();
    if (getenv("LSG_PLAN_DUMP")) {  // diagnostics: the plan on stderr
        for (size_t pi = 0; pi < plan.passes.size(); ++pi) {
            const PassDesc& pd = plan.passes[pi];
            std::fprintf(stderr, "pass %zu: K=%d L=%d hi=[", pi, pd.K, pd.L);
            for (int j = 0; j < pd.K - pd.L; ++j) std::fprintf(stderr, "%s%d", j ? "," : "", pd.hi[j]);
            std::fprintf(stderr, "] ops=%d blocks=%d\n", pd.nops, pd.nblocks);
            for (int bi = pd.first_block; bi < pd.first_block + pd.nblocks; ++bi) {
                const BlockDesc& b = plan.blocks[bi];
                std::fprintf(stderr, "  block u=%d generic=%d bits=[%d,%d,%d,%d] ops:", b.u, b.generic, b.bits[0],
                             b.bits[1], b.bits[2], b.bits[3]);
                for (int o = b.first; o < b.first + b.nops; ++o) {
                    const TileOp& t = plan.ops[pd.first_op + o];
                    std::fprintf(stderr, " %d/%d@%d", t.kind, t.k, t.tmpl);
                }
                std::fprintf(stderr, "\n");
            }
        }
    }
    return LSG_OK;
}

int lsg_program_free(lsg_program p) {
    clear_error();
    program_destroy(p);
    return LSG_OK;
}

}  // extern "C"

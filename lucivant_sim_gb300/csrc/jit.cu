// Passes specialized at run time. A planned program's passes are written out as CUDA source —
// for every register block its tile bits, group offsets, operators and data offsets as
// compile-time constants, the operators as a straight-line sequence of the register-block
// functions of tile.cuh — compiled once with NVRTC for sm_103a and launched through the driver
// API on the register's stream. The interpreter (k_tile_pipe) decodes each operator at run time:
// a dispatch per operator and group, register moves where the cases merge, address arithmetic for
// run-time bit positions. Specialized passes keep only the loads, the arithmetic and the stores.
//
// NVRTC and the driver entry points are looked up at run time (dlopen, cudaGetDriverEntryPoint):
// the library loads without them and programs fall back to the interpreter when they are
// missing. Compiled modules are cached by their source for the life of the process.
#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "jit.cuh"
#include "jit_headers.inc"  // generated by build.py: the device headers as strings

namespace lsg {
namespace {

struct Nvrtc {
    bool ok = false;
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

const Nvrtc& nvrtc() {
    static Nvrtc n = [] {
        Nvrtc r;
        void* h = nullptr;
        for (const char* name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) return r;
        r.create = reinterpret_cast<decltype(r.create)>(dlsym(h, "nvrtcCreateProgram"));
        r.compile = reinterpret_cast<decltype(r.compile)>(dlsym(h, "nvrtcCompileProgram"));
        r.log_size = reinterpret_cast<decltype(r.log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
        r.log = reinterpret_cast<decltype(r.log)>(dlsym(h, "nvrtcGetProgramLog"));
        r.cubin_size = reinterpret_cast<decltype(r.cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
        r.cubin = reinterpret_cast<decltype(r.cubin)>(dlsym(h, "nvrtcGetCUBIN"));
        r.destroy = reinterpret_cast<decltype(r.destroy)>(dlsym(h, "nvrtcDestroyProgram"));
        r.ok = r.create && r.compile && r.log_size && r.log && r.cubin_size && r.cubin && r.destroy;
        return r;
    }();
    return n;
}

struct Driver {
    bool ok = false;
    CUresult (*module_load)(CUmodule*, const void*) = nullptr;
    CUresult (*get_function)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                       void**, void**) = nullptr;
    CUresult (*set_attribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
    CUresult (*module_unload)(CUmodule) = nullptr;
    CUresult (*get_attribute)(int*, CUfunction_attribute, CUfunction) = nullptr;  // optional
    CUresult (*encode)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                       const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                       CUtensorMapL2promotion, CUtensorMapFloatOOBfill) = nullptr;  // optional
};

const Driver& driver() {
    static Driver d = [] {
        Driver r;
        auto get = [](const char* sym, void** fp) {
            cudaDriverEntryPointQueryResult q;
            return cudaGetDriverEntryPointByVersion(sym, fp, 12000, cudaEnableDefault, &q) == cudaSuccess &&
                   q == cudaDriverEntryPointSuccess && *fp;
        };
        r.ok = get("cuModuleLoadData", reinterpret_cast<void**>(&r.module_load)) &&
               get("cuModuleGetFunction", reinterpret_cast<void**>(&r.get_function)) &&
               get("cuLaunchKernel", reinterpret_cast<void**>(&r.launch)) &&
               get("cuFuncSetAttribute", reinterpret_cast<void**>(&r.set_attribute)) &&
               get("cuOccupancyMaxActiveBlocksPerMultiprocessor", reinterpret_cast<void**>(&r.occupancy)) &&
               get("cuModuleUnload", reinterpret_cast<void**>(&r.module_unload));
        if (!get("cuTensorMapEncodeTiled", reinterpret_cast<void**>(&r.encode))) r.encode = nullptr;
        if (!get("cuFuncGetAttribute", reinterpret_cast<void**>(&r.get_attribute))) r.get_attribute = nullptr;
        cudaGetLastError();
        return r;
    }();
    return d;
}

const char* type_name(int precision) {
    switch (precision) {
        case LSG_C128: return "lsg::Cx<double>";
        case LSG_C64: return "lsg::Cx<float>";
        case LSG_R64: return "double";
        case LSG_RD: return "lsg::DF";
        default: return "float";
    }
}

// One register-block operator as a call with compile-time positions; false for kinds that
// specialized passes do not take (mixtures and other trajectory operators). `packed`: the
// operands are real32 group pairs packed in 64-bit registers (tile.cuh F2, rp_* operators).
bool op_call(std::ostringstream& o, const TileOp& t, int U, const char* T, int at, bool packed = false) {
    const int c = t.tmpl;
    // data operators: rb_name<T, U, ...> or, packed, rp_name<U, ...>; renames: rb_name<T or F2, U, ...>
    auto name = [&](const char* fn, bool data_op) {
        if (packed && data_op) o << "rp_" << fn << "<" << U;
        else o << "rb_" << fn << "<" << (packed ? "lsg::F2" : T) << ", " << U;
    };
    auto two = [&](const char* fn, int base, bool data_op = true, int extra = 0) {
        const int r = c - base;
        name(fn, data_op);
        o << ", " << r / 4 << ", " << r % 4;
        if (extra) o << ", " << extra;
        o << ">";
    };
    auto one = [&](const char* fn, int base, bool data_op = true) {
        name(fn, data_op);
        o << ", " << (c - base) << ">";
    };
    bool data = true;
    if (c >= kT_DENSE1 && c < kT_DENSE1 + 4) one("dense1", kT_DENSE1);
    else if (c >= kT_DENSE2 && c < kT_DENSE2 + 16) two("dense2", kT_DENSE2);
    else if (c >= kT_TPD2 && c < kT_TPD2 + 16) two("tpd2", kT_TPD2, true, t.zmask);  // zero terms left out
    else if (c >= kT_PERM1 && c < kT_PERM1 + 4) one("perm1", kT_PERM1);
    else if (c >= kT_PERM2 && c < kT_PERM2 + 16) two("perm2", kT_PERM2);
    else if (packed && ((c >= kT_DEPOL1 && c < kT_DEPOL1 + 16) || c == kT_DEPOL2)) return false;  // complex only
    else if (c >= kT_DEPOL1 && c < kT_DEPOL1 + 16) two("depol1", kT_DEPOL1);
    else if (c == kT_DEPOL2 && U == 4) o << "rb_depol2<" << T << ">";
    else if (c == kT_DIAGB) name("diagb", true), o << ">";
    else if (c == kT_SCALE) name("scale", true), o << ">";
    else if (c == kT_DENSEB && !packed) name("denseb", true), o << ">";
    else if (c >= kT_X1 && c < kT_X1 + 4) one("x", kT_X1, false), data = false;
    else if (c >= kT_CX && c < kT_CX + 16) two("cx", kT_CX, false), data = false;
    else if (c >= kT_SWAP && c < kT_SWAP + 16) two("swap", kT_SWAP, false), data = false;
    else return false;
    const std::string v = at ? "v + " + std::to_string(at) : std::string("v");
    if (data) o << "(" << v << ", data + " << t.data << "LL + member * " << t.stride << "LL);\n";
    else o << "(" << v << ");\n";
    return true;
}

constexpr int kComputeHost = 256;  // compute threads of a pipelined pass CTA (tile.cuh kCompute)

// The 32-bit registers a thread may spend on its blocks' amplitudes at `ctas` CTAs per SM.
int state_reg_budget(int ctas) { return ctas >= 3 ? 32 : ctas == 2 ? 64 : 128; }

// A rename of tile offsets: the register-block renames (X, CX, SWAP codes) lifted to tile bits.
// Each is an involution x -> x ^ (bit a of x) << b (CX), a swap of bits a and b, or x ^ 1 << a (X).
struct Rename {
    int kind;  // 0 CX (control a, target b), 1 SWAP, 2 X (bit a)
    int a, b;
    uint32_t apply(uint32_t x) const {
        if (kind == 0) return x ^ (((x >> a) & 1u) << b);
        if (kind == 1) {
            const uint32_t d = ((x >> a) ^ (x >> b)) & 1u;
            return x ^ ((d << a) | (d << b));
        }
        return x ^ (1u << a);
    }
    // the bits that can be set after this rename when `may` can be set before it
    uint32_t may(uint32_t m) const {
        if (kind == 0) return m | (((m >> a) & 1u) << b);
        if (kind == 1) {
            const uint32_t ba = (m >> a) & 1u, bb = (m >> b) & 1u;
            return (m & ~((1u << a) | (1u << b))) | (ba << b) | (bb << a);
        }
        return m | (1u << a);
    }
    uint32_t bits() const { return kind == 2 ? 1u << a : (1u << a) | (1u << b); }
    void emit(std::ostringstream& o, const char* var) const {
        if (kind == 0) o << "      " << var << " ^= ((" << var << " >> " << a << ") & 1u) << " << b << ";\n";
        else if (kind == 1)
            o << "      { const uint32_t d = ((" << var << " >> " << a << ") ^ (" << var << " >> " << b << ")) & 1u; " << var
              << " ^= (d << " << a << ") | (d << " << b << "); }\n";
        else o << "      " << var << " ^= " << (1u << a) << "u;\n";
    }
};

// The renames of a block made only of X/CX/SWAP operators, in program order, or false.
bool pure_renames(const Plan& plan, const PassDesc& pd, const BlockDesc& b, std::vector<Rename>* out) {
    if (b.nops == 0) return false;
    for (int k = b.first; k < b.first + b.nops; ++k) {
        const int c = plan.ops[pd.first_op + k].tmpl;
        if (c >= kT_X1 && c < kT_X1 + 4) out->push_back({2, b.bits[c - kT_X1], 0});
        else if (c >= kT_CX && c < kT_CX + 16) out->push_back({0, b.bits[(c - kT_CX) / 4], b.bits[(c - kT_CX) % 4]});
        else if (c >= kT_SWAP && c < kT_SWAP + 16) out->push_back({1, b.bits[(c - kT_SWAP) / 4], b.bits[(c - kT_SWAP) % 4]});
        else return false;
    }
    return true;
}

// The shared-memory layout of tiles moved by swizzled tensor copies (common.cuh Tmap):
// element offset x is stored at S(x) = x ^ (((x >> row) & 7) << unit), the 128-byte swizzle in
// elements (16-byte units `unit` bits up, 128-byte rows `row` bits up). S is linear over GF(2):
// S(a ^ b) = S(a) ^ S(b), so a group's runtime base and its constant offsets swizzle apart.
struct Swizzle {
    bool on = false;
    int unit = 0, row = 0;
    static Swizzle for_elem(bool on, int elem_bytes) {
        Swizzle z;
        z.on = on;
        int lg = 0;
        while ((1 << lg) < elem_bytes) ++lg;
        z.unit = 4 - lg;
        z.row = 7 - lg;
        return z;
    }
    uint32_t apply(uint32_t x) const { return on ? x ^ (((x >> row) & 7u) << unit) : x; }
    uint32_t may(uint32_t m) const { return on ? m | (((m >> row) & 7u) << unit) : m; }
};

// One register block as generated: its access shape, and the renames folded into its loads
// (applied to the load addresses, last rename first) and stores (in program order).
struct BlockGen {
    const BlockDesc* b = nullptr;
    int U = 0, n = 0, groups = 0, W = 1, run = 1, elem_bytes = 4;
    // the bits of the group loop index a warp's lanes drive (5, ascending): chosen so that the
    // block's shared-memory accesses of one warp need the fewest wavefronts
    int lane_bits[5] = {0, 1, 2, 3, 4};
    std::vector<uint32_t> off;
    uint32_t vec_bits = 0;  // tile bits inside one shared-memory access (renames must keep them)
    std::vector<Rename> load_map, store_map;
    // A folded map moves elements between groups: every group must be in registers (one group
    // per compute thread) before any is stored, so the block takes one barrier between its loads
    // and its stores, and folding needs at most one group (pair) per compute thread.
    bool takes(const std::vector<Rename>& rn) const {
        if (groups / W > kComputeHost) return false;
        for (const Rename& r : rn)
            if (r.bits() & vec_bits) return false;
        return true;
    }
    bool folded() const { return !load_map.empty() || !store_map.empty(); }
};

BlockGen block_gen(const BlockDesc& b, const PassDesc& pd, int elem_bytes, int ctas, const Swizzle& sw) {
    BlockGen g;
    g.b = &b;
    g.U = b.u, g.n = 1 << b.u, g.groups = 1 << (pd.K - b.u);
    g.elem_bytes = elem_bytes;
    // Two groups per thread when tile bit 0 is not a block bit: the pair (tile bit 0 = 0, 1)
    // moves as one wider shared-memory access and every operator's coefficients, loaded once,
    // serve both groups (the two calls read the same addresses). Only when there are at least as
    // many pairs as compute threads: with fewer, half the threads would wait at the block's
    // barrier (a 32 KB tile of 8-byte elements holds 256 groups of 16).
    g.W = (b.sorted[0] != 0 && g.groups >= 2 * kComputeHost && 2 * g.n * elem_bytes / 4 <= state_reg_budget(ctas)) ? 2 : 1;
    if (sw.on && sw.unit == 0) g.W = 1;  // a pair must share a 16-byte unit: the swizzle moves whole units
    g.run = g.W == 2 ? 1 : std::min(std::max((int)b.vec, 1), std::max(1, 16 / elem_bytes));
    if (sw.on) g.run = std::min(g.run, 1 << sw.unit);
    g.vec_bits = g.W == 2 ? 1u : g.run == 4 ? 3u : g.run == 2 ? 1u : 0u;
    g.off.resize(g.n);
    for (int e = 0; e < g.n; ++e) {
        uint32_t a = 0;
        for (int i = 0; i < g.U; ++i)
            if ((e >> (g.U - 1 - i)) & 1) a |= 1u << b.bits[i];
        g.off[e] = a;
    }
    return g;
}

// The address expressions of a block's elements under a folded rename map and the tile's
// swizzle: the runtime part (the group base, renamed, swizzled) in `var`, a constant per element,
// joined by + where they cannot share a bit (an immediate offset) and by ^ where they can.
std::vector<std::string> mapped_addresses(std::ostringstream& o, const BlockGen& g, const std::vector<Rename>& map,
                                          const char* var, uint32_t tile_mask, const Swizzle& sw) {
    std::vector<std::string> addr(g.n);
    if (map.empty() && !sw.on) {
        for (int e = 0; e < g.n; ++e) addr[e] = "base + " + std::to_string(g.off[e]) + "u";
        return addr;
    }
    uint32_t block_bits = 0;
    for (int i = 0; i < g.U; ++i) block_bits |= 1u << g.b->bits[i];
    uint32_t may = tile_mask & ~block_bits & ~(g.W == 2 ? 1u : 0u) & ~g.vec_bits;
    o << "      uint32_t " << var << " = base;\n";
    uint32_t zero = 0;
    for (const Rename& r : map) {
        r.emit(o, var);
        may = r.may(may);
        zero = r.apply(zero);
    }
    if (sw.on) {
        o << "      " << var << " ^= ((" << var << " >> " << sw.row << ") & 7u) << " << sw.unit << ";\n";
        may = sw.may(may);
    }
    for (int e = 0; e < g.n; ++e) {
        uint32_t c = g.off[e];
        for (const Rename& r : map) c = r.apply(c);
        c = sw.apply(c ^ zero);  // the map is affine: map(base ^ off) = map(base) ^ map(off) ^ map(0)
        addr[e] = std::string(var) + ((c & may) ? " ^ " : " + ") + std::to_string(c) + "u";
    }
    return addr;
}

// The group loop index with its low five bits (the lane) moved to the positions in `lane` and
// the other bits, in order, to the remaining positions below `m` bits: a bijection of [0, 2^m).
uint32_t lane_permute(uint32_t g, const int* lane, int m) {
    uint32_t out = 0, lanes = 0;
    for (int i = 0; i < 5; ++i) {
        out |= ((g >> i) & 1u) << lane[i];
        lanes |= 1u << lane[i];
    }
    int src = 5;
    for (int t = 0; t < m; ++t)
        if (!((lanes >> t) & 1u)) out |= ((g >> src++) & 1u) << t;
    return out;
}

// Element addresses of one group (base = the group's first element) under a folded rename map
// and the swizzle, as mapped_addresses emits them.
void group_addresses(const BlockGen& g, uint32_t base, const std::vector<Rename>& map, uint32_t tile_mask,
                     const Swizzle& sw, std::vector<uint32_t>& out) {
    out.resize(g.n);
    if (map.empty() && !sw.on) {
        for (int e = 0; e < g.n; ++e) out[e] = base + g.off[e];
        return;
    }
    uint32_t block_bits = 0;
    for (int i = 0; i < g.U; ++i) block_bits |= 1u << g.b->bits[i];
    uint32_t may = tile_mask & ~block_bits & ~(g.W == 2 ? 1u : 0u) & ~g.vec_bits;
    uint32_t var = base, zero = 0;
    for (const Rename& r : map) {
        var = r.apply(var);
        may = r.may(may);
        zero = r.apply(zero);
    }
    if (sw.on) {
        var = sw.apply(var);
        may = sw.may(may);
    }
    for (int e = 0; e < g.n; ++e) {
        uint32_t c = g.off[e];
        for (const Rename& r : map) c = r.apply(c);
        c = sw.apply(c ^ zero);
        out[e] = (c & may) ? (var ^ c) : (var + c);
    }
}

// Shared-memory wavefronts of one warp's accesses (lane i at byte address addr[i], `bytes` wide):
// phases of 128 / bytes lanes; in each, the most distinct 4-byte words any bank must serve.
int warp_wavefronts(const uint32_t* addr, int bytes) {
    const int per = std::max(1, 128 / std::max(bytes, 4));
    int total = 0;
    for (int p0 = 0; p0 < 32; p0 += per) {
        uint32_t words[32][8];
        int count[32] = {0};
        int worst = 1;
        for (int l = p0; l < p0 + per && l < 32; ++l)
            for (int w = 0; w < std::max(bytes, 4) / 4; ++w) {
                const uint32_t word = addr[l] / 4 + (uint32_t)w;
                const int bank = (int)(word & 31u);
                bool seen = false;
                for (int k = 0; k < count[bank] && !seen; ++k) seen = words[bank][k] == word;
                if (!seen && count[bank] < 8) {
                    words[bank][count[bank]++] = word;
                    worst = std::max(worst, count[bank]);
                }
            }
        total += worst;
    }
    return total;
}

// Wavefronts of one warp's loads and stores of a block (the first warp of the loop, lanes driving
// the index bits in `lane`).
int block_wavefronts(const BlockGen& g, const int* lane, int m, uint32_t tile_mask, const Swizzle& sw) {
    const int bytes = (g.W == 2 ? 2 : g.run) * g.elem_bytes;
    std::vector<uint32_t> ld[32], st[32];
    for (int l = 0; l < 32; ++l) {
        const uint32_t G = lane_permute((uint32_t)l, lane, m) << (g.W == 2 ? 1 : 0);
        uint32_t base = 0;
        for (int i = 0; i <= g.U; ++i) base |= (G << i) & g.b->dep[i];
        group_addresses(g, base, g.load_map, tile_mask, sw, ld[l]);
        group_addresses(g, base, g.store_map, tile_mask, sw, st[l]);
    }
    int total = 0;
    uint32_t a[32];
    for (int e = 0; e < g.n; e += g.run) {
        for (int l = 0; l < 32; ++l) a[l] = ld[l][e] * (uint32_t)g.elem_bytes;
        total += warp_wavefronts(a, bytes);
        for (int l = 0; l < 32; ++l) a[l] = st[l][e] * (uint32_t)g.elem_bytes;
        total += warp_wavefronts(a, bytes);
    }
    return total;
}

// Pick the five index bits the lanes drive (a 5-subset of the loop index's bits, ascending) with
// the fewest wavefronts; the lowest five when nothing is better.
void choose_lane_bits(BlockGen& g, uint32_t tile_mask, const Swizzle& sw) {
    int m = 0;
    while ((1 << m) < g.groups / g.W) ++m;
    if (m <= 5) return;
    int best[5] = {0, 1, 2, 3, 4};
    int best_cost = block_wavefronts(g, best, m, tile_mask, sw);
    int c[5];
    for (c[0] = 0; c[0] < m; ++c[0])
        for (c[1] = c[0] + 1; c[1] < m; ++c[1])
            for (c[2] = c[1] + 1; c[2] < m; ++c[2])
                for (c[3] = c[2] + 1; c[3] < m; ++c[3])
                    for (c[4] = c[3] + 1; c[4] < m; ++c[4]) {
                        const int cost = block_wavefronts(g, c, m, tile_mask, sw);
                        if (cost < best_cost) {
                            best_cost = cost;
                            std::copy(c, c + 5, best);
                        }
                    }
    std::copy(best, best + 5, g.lane_bits);
}

// The generated expression of lane_permute(g) (constant positions; runs of bits move together).
std::string lane_permute_expr(const BlockGen& g, int m) {
    int target[32];
    uint32_t lanes = 0;
    for (int i = 0; i < 5; ++i) {
        target[i] = g.lane_bits[i];
        lanes |= 1u << g.lane_bits[i];
    }
    int src = 5;
    for (int t = 0; t < m; ++t)
        if (!((lanes >> t) & 1u)) target[src++] = t;
    std::ostringstream e;
    bool first = true;
    for (int j = 0; j < m;) {
        int k = j + 1;
        while (k < m && target[k] == target[k - 1] + 1) ++k;
        const uint32_t mask = (1u << (k - j)) - 1u;
        e << (first ? "" : " | ") << "(((uint32_t(g) >> " << j << ") & " << mask << "u) << " << target[j] << ")";
        first = false;
        j = k;
    }
    return e.str();
}

void emit_block(std::ostringstream& o, const BlockGen& g, const Plan& plan, const PassDesc& pd, const char* T,
                const Swizzle& sw, bool packed, bool* ok) {
    const BlockDesc& b = *g.b;
    const bool pk = packed && g.W == 2;  // the group pair in packed 64-bit registers (real32)
    const uint32_t tile_mask = pd.K >= 32 ? ~0u : ((1u << pd.K) - 1u);
    const bool fold = g.folded();
    if (fold)  // one group (pair) per thread; threads past the last group only join the barriers
        o << "    cbar();\n    {\n      const int g = threadIdx.x;\n      const bool act = g < " << g.groups / g.W << ";\n";
    else
        o << "    cbar();\n    for (int g = threadIdx.x; g < " << g.groups / g.W << "; g += kCompute) {\n";
    int m = 0;
    while ((1 << m) < g.groups / g.W) ++m;
    const bool moved = m > 5 && !(g.lane_bits[0] == 0 && g.lane_bits[1] == 1 && g.lane_bits[2] == 2 &&
                                  g.lane_bits[3] == 3 && g.lane_bits[4] == 4);
    if (moved)
        o << "      const uint32_t G = (" << lane_permute_expr(g, m) << ")" << (g.W == 2 ? " << 1" : "") << ";\n";
    else
        o << "      const uint32_t G = uint32_t(g)" << (g.W == 2 ? " << 1" : "") << ";\n";
    o << "      const uint32_t base =";
    for (int i = 0; i <= g.U; ++i) o << (i ? " |" : "") << " ((G << " << i << ") & " << b.dep[i] << "u)";
    if (pk) o << ";\n      lsg::F2 v[" << g.n << "];\n";
    else o << ";\n      " << T << " v[" << g.n * g.W << "];\n";
    const std::vector<std::string> la = mapped_addresses(o, g, g.load_map, "lb", tile_mask, sw);
    if (fold) o << "      if (act) {\n";
    for (int e = 0; e < g.n; e += g.run) {
        if (pk)
            o << "      v[" << e << "] = ld_f2(tile + (" << la[e] << "));\n";
        else if (g.W == 2)
            o << "      ld_split<" << T << ">(tile + (" << la[e] << "), v[" << e << "], v[" << g.n + e << "]);\n";
        else
            o << "      ld_run<" << T << ", " << g.run << ">(tile + (" << la[e] << "), v + " << e << ");\n";
    }
    for (int k = b.first; k < b.first + b.nops; ++k)
        for (int w = 0; w < (pk ? 1 : g.W); ++w) {
            o << "      ";
            if (!op_call(o, plan.ops[pd.first_op + k], g.U, T, w * g.n, pk)) {
                *ok = false;
                return;
            }
        }
    if (fold) o << "      }\n      cbar();  // every group is in registers: the renamed stores may land in any group\n      if (act) {\n";
    const std::vector<std::string> sa = mapped_addresses(o, g, g.store_map, "sb", tile_mask, sw);
    for (int e = 0; e < g.n; e += g.run) {
        if (pk)
            o << "      st_f2(tile + (" << sa[e] << "), v[" << e << "]);\n";
        else if (g.W == 2)
            o << "      st_split<" << T << ">(tile + (" << sa[e] << "), v[" << e << "], v[" << g.n + e << "]);\n";
        else
            o << "      st_run<" << T << ", " << g.run << ">(tile + (" << sa[e] << "), v + " << e << ");\n";
    }
    if (fold) o << "      }\n";
    o << "    }\n";
}

std::string pass_source(const Plan& plan, size_t pi, int precision, int elem_bytes, int ctas, bool swz, bool packed) {
    const PassDesc& pd = plan.passes[pi];
    const char* T = type_name(precision);
    const Swizzle sw = Swizzle::for_elem(swz, elem_bytes);
    // Blocks made only of renames move no arithmetic: they fold into the neighbouring block's
    // store addresses (or the next block's load addresses) unless they touch the bits inside
    // that block's vector accesses, saving a shared-memory round trip and a barrier each.
    std::vector<BlockGen> gens, held;
    std::vector<Rename> pending;
    for (int bi = pd.first_block; bi < pd.first_block + pd.nblocks; ++bi) {
        const BlockDesc& b = plan.blocks[bi];
        if (b.generic) return "";
        BlockGen g = block_gen(b, pd, elem_bytes, ctas, sw);
        std::vector<Rename> rn;
        if (pure_renames(plan, pd, b, &rn)) {
            if (held.empty() && !gens.empty() && gens.back().takes(rn)) {
                gens.back().store_map.insert(gens.back().store_map.end(), rn.begin(), rn.end());
                continue;
            }
            held.push_back(g);
            pending.insert(pending.end(), rn.begin(), rn.end());
            continue;
        }
        if (!held.empty()) {
            if (g.takes(pending)) g.load_map.assign(pending.rbegin(), pending.rend());
            else gens.insert(gens.end(), held.begin(), held.end());
            held.clear();
            pending.clear();
        }
        gens.push_back(g);
    }
    gens.insert(gens.end(), held.begin(), held.end());
    {
        const char* env = getenv("LSG_LANE_BITS");  // 0: lanes drive the lowest index bits (diagnostics)
        if (!(env && env[0] == '0')) {
            const uint32_t tile_mask = pd.K >= 32 ? ~0u : ((1u << pd.K) - 1u);
            for (BlockGen& g : gens) choose_lane_bits(g, tile_mask, sw);
        }
    }
    std::ostringstream o;
    o << "struct Body" << pi << " {\n  static __device__ __forceinline__ void run(" << T << "* tile, const " << T
      << "* __restrict__ data, long long member) {\n";
    bool ok = true;
    for (const BlockGen& g : gens) {
        emit_block(o, g, plan, pd, T, sw, packed && precision == LSG_R32, &ok);
        if (!ok) return "";
    }
    o << "    cbar();\n  }\n};\n";
    return o.str();
}

std::mutex g_mu;
std::map<std::string, std::shared_ptr<JitPasses>> g_cache;
std::vector<std::string> g_order;  // cache keys, oldest first
// programs of that many shapes keep their modules cached (LSG_JIT_CACHE_MAX, default 64)
size_t jit_cache_max() {
    const char* env = getenv("LSG_JIT_CACHE_MAX");
    return env ? (size_t)std::max(1, atoi(env)) : 64;
}
bool g_exiting = false;            // set at exit: the driver may be gone, modules are not unloaded

}  // namespace

JitPasses::~JitPasses() {
    if (g_exiting || !driver().module_unload) return;
    for (void* m : modules) driver().module_unload(static_cast<CUmodule>(m));
}

int jit_mode() {
    const char* env = getenv("LSG_JIT");
    if (!env || !env[0]) return 2;
    return env[0] == '0' ? 0 : 1;
}

bool jit_packed(int precision) {
    if (precision != LSG_R32) return false;
    const char* env = getenv("LSG_FFMA2");
    return !(env && env[0] == '0');
}

bool jit_wanted(int64_t bytes_per_run) {
    const int mode = jit_mode();
    if (mode != 2) return mode == 1;
    const char* env = getenv("LSG_JIT_MIN_BYTES");
    const int64_t min_bytes = env ? std::atoll(env) : (256ll << 30);
    return bytes_per_run >= min_bytes;
}

namespace {

// Pass i's body and kernel, or "" when the specializer does not take one of its blocks.
std::string pass_kernel_source(const Plan& plan, size_t i, int precision, int ctas, bool swz, bool packed) {
    const char* T = type_name(precision);
    const std::string body = pass_source(plan, i, precision, (int)lsg_elem_bytes(precision), ctas, swz, packed);
    if (body.empty()) return "";
    std::ostringstream o;
    o << body << "extern \"C\" __global__ void __launch_bounds__(" << kPipeThreadsHost << ", " << ctas
      << ") lsg_pass_" << i << "(" << T << "* state, long long me, const PassDesc* pg, const " << T
      << "* data, long long tpm, long long total, int* status, const __grid_constant__ lsg::Tmap tmap) {\n  pipe_kernel<"
      << T << ", Body" << i << ", " << (swz ? "true" : "false") << ">(state, me, pg, data, tpm, total, status, &tmap);\n}\n";
    return o.str();
}

const char* const kPrelude = "#include \"tile.cuh\"\nusing namespace lsg;\n";

// One translation unit to a cubin (empty on failure; the log into `log`, or on stderr with
// LSG_JIT_LOG).
std::vector<char> compile_unit(const std::string& source, std::string* log_out = nullptr) {
    const Nvrtc& rt = nvrtc();
    std::vector<char> cubin;
    nvrtcProgram prog;
    if (rt.create(&prog, source.c_str(), "lsg_passes.cu", kJitHeaderCount, kJitHeaderSources, kJitHeaderNames) !=
        NVRTC_SUCCESS)
        return cubin;
    // -default-device: the public header's host declarations are harmless device ones here
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device"};
    const nvrtcResult cr = rt.compile(prog, 3, opts);
    size_t bytes = 0;
    if (cr == NVRTC_SUCCESS && rt.cubin_size(prog, &bytes) == NVRTC_SUCCESS && bytes) {
        cubin.resize(bytes);
        if (rt.cubin(prog, cubin.data()) != NVRTC_SUCCESS) cubin.clear();
    } else if (log_out || getenv("LSG_JIT_LOG")) {
        size_t n = 0;
        rt.log_size(prog, &n);
        std::string log(n, '\0');
        rt.log(prog, &log[0]);
        if (log_out) *log_out = log;
        else std::fprintf(stderr, "pass specialization failed:\n%s\n", log.c_str());
    }
    rt.destroy(&prog);
    return cubin;
}

}  // namespace

int jit_compile_check(const std::string& source) {
    if (!nvrtc().ok) return fail(LSG_E_STATE, "NVRTC (libnvrtc.so.13) is not available");
    std::string log;
    if (compile_unit(source, &log).empty()) return fail(LSG_E_ARG, "specialized passes do not compile: %.900s", log.c_str());
    return LSG_OK;
}

bool jit_swizzle_fits(const Plan& plan, size_t elem_bytes, int64_t register_bytes) {
    const char* env = getenv("LSG_SWIZZLE");
    if (env && env[0] == '0') return false;
    if (register_bytes <= 0 || register_bytes % 1024 != 0 || (register_bytes >> 7) >= (1ll << 31)) return false;
    for (const PassDesc& pd : plan.passes) {
        // chunks of 512 bytes move in pairs (1 KB boxes), larger ones in whole 1 KB swizzle atoms
        const size_t chunk = elem_bytes << pd.L;
        if (chunk < 512 || chunk % 512 != 0 || pd.K <= pd.L) return false;
        if (chunk == 512 && ((elem_bytes << pd.hi[0]) % 1024 != 0 || (register_bytes / (elem_bytes << pd.hi[0])) >= (1ll << 31)))
            return false;
    }
    return true;
}

std::string jit_source(const Plan& plan, int precision, int ctas, bool swz, bool packed) {
    std::string src = kPrelude;
    for (size_t i = 0; i < plan.passes.size(); ++i) {
        const std::string k = pass_kernel_source(plan, i, precision, ctas, swz, packed);
        if (k.empty()) return "";  // a pass the specializer does not take: interpret them all
        src += k;
    }
    return src;
}

namespace {

// A loaded pass kernel: its function, resident CTAs per SM and local memory per thread (spills).
struct Loaded {
    void* fn = nullptr;
    int per_sm = 1;
    int local = 0;
};

// LSG_JIT_SPILL: local bytes per thread above which a pass compiled for three CTAs per SM is
// rebuilt for two (default 64; 0 or less: never).
int jit_spill_bytes() {
    const char* env = getenv("LSG_JIT_SPILL");
    return env && env[0] ? atoi(env) : 64;
}

// Compile kernels[i] for every i in `which` (passes are independent translation units: compiled
// in parallel, in chunks of about equal source length, NVRTC programs on concurrent host threads),
// load the modules (appended to `modules`) and fill out[i]. False on any failure.
bool compile_load(const std::vector<std::string>& kernels, const std::vector<size_t>& which, const Plan& plan,
                  size_t eb, bool swz, std::vector<Loaded>& out, std::vector<void*>& modules) {
    const Driver& drv = driver();
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nchunks = std::min<size_t>({which.size(), (size_t)hw, 16});
    if (nchunks == 0) return true;
    std::vector<std::string> units(nchunks, kPrelude);
    std::vector<std::vector<size_t>> members(nchunks);
    std::vector<size_t> load(nchunks, 0);
    for (size_t i : which) {
        const size_t c = std::min_element(load.begin(), load.end()) - load.begin();
        units[c] += kernels[i];
        members[c].push_back(i);
        load[c] += kernels[i].size();
    }
    std::vector<std::vector<char>> cubins(nchunks);
    std::vector<std::thread> workers;
    for (size_t c = 1; c < nchunks; ++c) workers.emplace_back([&, c] { cubins[c] = compile_unit(units[c]); });
    cubins[0] = compile_unit(units[0]);
    for (std::thread& w : workers) w.join();
    bool ok = true;
    for (size_t c = 0; c < nchunks && ok; ++c) {
        CUmodule mod;
        ok = !cubins[c].empty() && drv.module_load(&mod, cubins[c].data()) == CUDA_SUCCESS;
        if (ok) modules.push_back(mod);
        for (size_t j = 0; j < members[c].size() && ok; ++j) {
            const size_t i = members[c][j];
            const std::string name = "lsg_pass_" + std::to_string(i);
            CUfunction f;
            const size_t smem = 2 * (eb << plan.passes[i].K) + (swz ? 1024 : 0);  // the two-tile ring, aligned
            ok = drv.get_function(&f, mod, name.c_str()) == CUDA_SUCCESS &&
                 drv.set_attribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem) == CUDA_SUCCESS &&
                 drv.occupancy(&out[i].per_sm, f, kPipeThreadsHost, smem) == CUDA_SUCCESS;
            out[i].fn = f;
            if (ok && drv.get_attribute && drv.get_attribute(&out[i].local, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, f) != CUDA_SUCCESS)
                out[i].local = 0;
        }
    }
    return ok;
}

}  // namespace

std::shared_ptr<JitPasses> jit_build(const Plan& plan, int precision, int ctas, bool swz, bool packed) {
    const size_t np = plan.passes.size();
    if (np == 0) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    // The source is a function of the plan (its descriptors are value-initialised, padding
    // included), the precision, the CTAs per SM, the swizzle and the packing: the cache is keyed by their bytes,
    // so a program of a known shape (new data, same structure) skips source generation too.
    std::string key;
    {
        const int head[6] = {dev, precision, ctas, swz ? 1 : 0, packed ? 1 : 0, jit_spill_bytes()};
        const size_t sizes[3] = {plan.passes.size(), plan.ops.size(), plan.blocks.size()};
        key.reserve(sizeof(head) + sizeof(sizes) + sizes[0] * sizeof(PassDesc) + sizes[1] * sizeof(TileOp) +
                    sizes[2] * sizeof(BlockDesc));
        key.append(reinterpret_cast<const char*>(head), sizeof(head));
        key.append(reinterpret_cast<const char*>(sizes), sizeof(sizes));
        key.append(reinterpret_cast<const char*>(plan.passes.data()), sizes[0] * sizeof(PassDesc));
        key.append(reinterpret_cast<const char*>(plan.ops.data()), sizes[1] * sizeof(TileOp));
        key.append(reinterpret_cast<const char*>(plan.blocks.data()), sizes[2] * sizeof(BlockDesc));
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto hit = g_cache.find(key);
        if (hit != g_cache.end()) return hit->second;
    }
    std::vector<std::string> kernels(np);
    for (size_t i = 0; i < np; ++i) {
        kernels[i] = pass_kernel_source(plan, i, precision, ctas, swz, packed);
        if (kernels[i].empty()) break;  // a pass the specializer does not take: interpret them all
    }
    std::lock_guard<std::mutex> lock(g_mu);
    auto hit = g_cache.find(key);  // another thread may have built it meanwhile
    if (hit != g_cache.end()) return hit->second;
    const Nvrtc& rt = nvrtc();
    const Driver& drv = driver();
    static const bool at_exit = [] { return std::atexit([] { g_exiting = true; }) == 0; }();
    (void)at_exit;
    std::shared_ptr<JitPasses> out;
    const bool all = std::none_of(kernels.begin(), kernels.end(), [](const std::string& k) { return k.empty(); });
    if (all && rt.ok && drv.ok) {
        auto jp = std::make_shared<JitPasses>();
        jp->fns.resize(np);
        jp->per_sm.resize(np, 1);
        jp->swz = swz;
        const size_t eb = lsg_elem_bytes(precision);
        std::vector<size_t> every(np);
        for (size_t i = 0; i < np; ++i) every[i] = i;
        std::vector<Loaded> got(np);
        bool ok = compile_load(kernels, every, plan, eb, swz, got, jp->modules);
        // A pass whose registers spill at three CTAs per SM (local memory beyond the threshold:
        // with three CTAs' tiles in shared memory, spilled values overflow L1 to L2) is compiled
        // again for two, with more registers per thread, and keeps the smaller spill. Passes
        // compiled for two CTAs or fewer are kept: one CTA per SM leaves too few warps to cover
        // the memory latency of the lighter passes.
        const int spill = jit_spill_bytes();
        std::vector<size_t> again;
        for (size_t i = 0; ok && spill > 0 && ctas >= 3 && i < np; ++i)
            if (got[i].local > spill) again.push_back(i);
        if (ok && !again.empty()) {
            std::vector<std::string> fewer(np);
            for (size_t i : again) fewer[i] = pass_kernel_source(plan, i, precision, ctas - 1, swz, packed);
            std::vector<Loaded> alt(np);
            if (compile_load(fewer, again, plan, eb, swz, alt, jp->modules))
                for (size_t i : again)
                    if (alt[i].local < got[i].local) got[i] = alt[i];
        }
        for (size_t i = 0; ok && i < np; ++i) jp->fns[i] = got[i].fn, jp->per_sm[i] = got[i].per_sm;
        if (ok) out = jp;
    }
    g_cache[key] = out;  // a failure is remembered too: the interpreter runs those programs
    g_order.push_back(key);
    if (g_order.size() > jit_cache_max()) {  // forget the oldest shape (its programs keep their modules)
        g_cache.erase(g_order.front());
        g_order.erase(g_order.begin());
    }
    return out;
}

int jit_launch(const JitPasses& jp, const Plan& plan, void* state, int64_t member_elems, const void* pass_dev,
               size_t pass_stride, const void* data, const std::vector<int64_t>& tiles_per_member, int64_t batch,
               int* status, size_t tile_bytes, cudaStream_t stream, cudaEvent_t* marks) {
    const Driver& drv = driver();
    int dev = 0, sms = 0;
    LSG_CUDA(cudaGetDevice(&dev));
    LSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = 2 * tile_bytes + (jp.swz ? 1024 : 0);
    // the register as rows of 128 bytes, copied in boxes with the 128-byte swizzle (tile.cuh
    // pipe_run): 2-D boxes of min(chunk, 16 KB) for chunks of 1 KB and more, one map per box
    // height; 3-D boxes pairing two 512-byte chunks that differ in register bit h = hi[0], one map
    // per h (rows of 128 bytes, blocks of 2^h elements). Unused without swizzle.
    const uint64_t eb = (uint64_t)(tile_bytes >> plan.passes[0].K);
    const uint64_t bytes = (uint64_t)member_elems * (uint64_t)batch * eb;
    std::map<uint32_t, CUtensorMap> maps;
    auto map_for = [&](const PassDesc& pd, CUtensorMap** out) -> int {
        const uint64_t chunk = eb << pd.L;
        const bool pair = chunk == 512;
        const uint32_t key = pair ? (0x80000000u | (uint32_t)pd.hi[0]) : (uint32_t)(std::min<uint64_t>(chunk, 16384) >> 7);
        auto it = maps.find(key);
        if (it == maps.end()) {
            CUtensorMap m;
            std::memset(&m, 0, sizeof(m));
            if (jp.swz) {
                if (!drv.encode) return fail(LSG_E_STATE, "cuTensorMapEncodeTiled is not available");
                const uint64_t block = pair ? eb << pd.hi[0] : 0;
                if (bytes % 1024 != 0 || (bytes >> 7) >= (1ull << 31) || (pair && (block % 1024 != 0 || bytes % block != 0)))
                    return fail(LSG_E_STATE, "a register of %llu bytes does not fit the swizzled tensor copies",
                                (unsigned long long)bytes);
                cuuint64_t dims[3] = {32, pair ? block >> 7 : bytes >> 7, pair ? bytes / block : 1};
                cuuint64_t strides[2] = {128, block};
                cuuint32_t box[3] = {32, pair ? 4u : key, 2};
                cuuint32_t estr[3] = {1, 1, 1};
                if (drv.encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT32, pair ? 3 : 2, state, dims, strides, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return fail(LSG_E_CUDA, "encoding the register's tensor map failed");
            }
            it = maps.emplace(key, m).first;
        }
        *out = &it->second;
        return LSG_OK;
    };
    for (size_t i = 0; i < plan.passes.size(); ++i) {
        CUtensorMap* map = nullptr;
        LSG_CHECK(map_for(plan.passes[i], &map));
        CUfunction f = reinterpret_cast<CUfunction>(jp.fns[i]);
        const int64_t total = tiles_per_member[i] * batch;
        const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(total, (int64_t)sms * std::max(jp.per_sm[i], 1)));
        const void* pg = static_cast<const unsigned char*>(pass_dev) + i * pass_stride;
        long long me = member_elems, tpm = tiles_per_member[i], tot = total;
        void* args[] = {&state, &me, &pg, &data, &tpm, &tot, &status, map};
        if (marks) LSG_CUDA(cudaEventRecord(marks[i], stream));
        if (drv.launch(f, (unsigned)grid, 1, 1, kPipeThreadsHost, 1, 1, (unsigned)smem, (CUstream)stream, args, nullptr) !=
            CUDA_SUCCESS)
            return fail(LSG_E_CUDA, "launching a specialized pass failed");
    }
    return LSG_OK;
}

}  // namespace lsg

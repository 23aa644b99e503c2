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
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "program.cuh"

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
    if (s.ptr) cudaFree(s.ptr);
    s.ptr = nullptr;
    s.bytes = 0;
    size_t want = std::max<size_t>(bytes, 4096);
    LSG_CUDA(cudaMalloc(&s.ptr, want));
    s.bytes = want;
    return LSG_OK;
}

void release(Scratch& s) {
    if (s.ptr) cudaFree(s.ptr);
    s.ptr = nullptr;
    s.bytes = 0;
}

// ------------------------------------------------------------------------ tile kernel

template <typename R>
struct Smem {
    // Cx<R> tile[1 << K] follows in dynamic shared memory
};

// Deposit the bits of x into the register positions listed in pos[0..n) (ascending).
__device__ __forceinline__ uint64_t deposit(uint64_t x, const int* pos, int n) {
    uint64_t out = 0;
    for (int j = 0; j < n; ++j) out |= ((x >> j) & 1ull) << pos[j];
    return out;
}

template <typename R, int KB>
__device__ __forceinline__ void op_matrix(Cx<R>* tile, int tbits, const TileOp& op, const Cx<R>* m) {
    constexpr int D = 1 << KB;
    uint64_t offs[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
#pragma unroll
        for (int i = 0; i < KB; ++i) o |= (uint64_t)((j >> (KB - 1 - i)) & 1) << op.lb[i];
        offs[j] = o;
    }
    const int groups = 1 << (tbits - KB);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        uint64_t base = spread((uint64_t)g, op.sorted, KB);
        Cx<R> v[D];
#pragma unroll
        for (int j = 0; j < D; ++j) v[j] = tile[base | offs[j]];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            Cx<R> acc;
#pragma unroll
            for (int c = 0; c < D; ++c) acc = cfma(m[r * D + c], v[c], acc);
            tile[base | offs[r]] = acc;
        }
    }
}

template <typename R, int KB>
__device__ __forceinline__ void op_perm(Cx<R>* tile, int tbits, const TileOp& op, const Cx<R>* m) {
    constexpr int D = 1 << KB;
    uint64_t offs[D];
    int src[D];
    Cx<R> ph[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
#pragma unroll
        for (int i = 0; i < KB; ++i) o |= (uint64_t)((j >> (KB - 1 - i)) & 1) << op.lb[i];
        offs[j] = o;
        ph[j] = m[j];
        src[j] = (int)m[D + j].re;
    }
    const int groups = 1 << (tbits - KB);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        uint64_t base = spread((uint64_t)g, op.sorted, KB);
        Cx<R> v[D];
#pragma unroll
        for (int j = 0; j < D; ++j) v[j] = tile[base | offs[j]];
#pragma unroll
        for (int r = 0; r < D; ++r) tile[base | offs[r]] = cmul(ph[r], v[src[r]]);
    }
}

template <typename R>
__device__ __forceinline__ void op_diag(Cx<R>* tile, int tbits, const TileOp& op, const Cx<R>* m) {
    const int n = 1 << tbits;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int j = 0;
        for (int b = 0; b < op.k; ++b) j = (j << 1) | ((i >> op.lb[b]) & 1);
        tile[i] = cmul(m[j], tile[i]);
    }
}

template <typename R>
__device__ __forceinline__ void op_scale(Cx<R>* tile, int tbits, const Cx<R>* m) {
    const int n = 1 << tbits;
    const Cx<R> f = m[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) tile[i] = cmul(f, tile[i]);
}

// (1-p) rho + (p/d) I (x) Tr_t(rho): k row bits then k column bits (k = 1 or 2).
template <typename R, int KQ>
__device__ __forceinline__ void op_depol(Cx<R>* tile, int tbits, const TileOp& op, const Cx<R>* m) {
    constexpr int KB = 2 * KQ;
    constexpr int D = 1 << KB;
    constexpr int d = 1 << KQ;
    uint64_t offs[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        uint64_t o = 0;
#pragma unroll
        for (int i = 0; i < KB; ++i) o |= (uint64_t)((j >> (KB - 1 - i)) & 1) << op.lb[i];
        offs[j] = o;
    }
    const R p = m[0].re;
    const R keep = R(1) - p;
    const R share = p / R(d);
    const int groups = 1 << (tbits - KB);
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        uint64_t base = spread((uint64_t)g, op.sorted, KB);
        Cx<R> tr;
#pragma unroll
        for (int t = 0; t < d; ++t) {
            Cx<R> v = tile[base | offs[(t << KQ) | t]];
            tr.re += v.re;
            tr.im += v.im;
        }
#pragma unroll
        for (int j = 0; j < D; ++j) {
            Cx<R> v = tile[base | offs[j]];
            Cx<R> o(v.re * keep, v.im * keep);
            if ((j >> KQ) == (j & (d - 1))) {
                o.re += share * tr.re;
                o.im += share * tr.im;
            }
            tile[base | offs[j]] = o;
        }
    }
}

template <typename R>
__device__ void run_ops(Cx<R>* tile, int tbits, const TileOp* __restrict__ ops, int nops,
                        const Cx<R>* __restrict__ data, int64_t member) {
    for (int o = 0; o < nops; ++o) {
        TileOp op = ops[o];
        const Cx<R>* m = data + op.data + member * op.stride;
        __syncthreads();
        switch (op.kind) {
            case LSG_OP_MATRIX:
                switch (op.k) {
                    case 1: op_matrix<R, 1>(tile, tbits, op, m); break;
                    case 2: op_matrix<R, 2>(tile, tbits, op, m); break;
                    case 3: op_matrix<R, 3>(tile, tbits, op, m); break;
                    case 4: op_matrix<R, 4>(tile, tbits, op, m); break;
                    case 5: op_matrix<R, 5>(tile, tbits, op, m); break;
                    default: break;
                }
                break;
            case LSG_OP_PERM:
                switch (op.k) {
                    case 1: op_perm<R, 1>(tile, tbits, op, m); break;
                    case 2: op_perm<R, 2>(tile, tbits, op, m); break;
                    case 3: op_perm<R, 3>(tile, tbits, op, m); break;
                    case 4: op_perm<R, 4>(tile, tbits, op, m); break;
                    case 5: op_perm<R, 5>(tile, tbits, op, m); break;
                    default: break;
                }
                break;
            case LSG_OP_DIAG: op_diag<R>(tile, tbits, op, m); break;
            case LSG_OP_DEPOL:
                if (op.k == 2) op_depol<R, 1>(tile, tbits, op, m);
                else op_depol<R, 2>(tile, tbits, op, m);
                break;
            case LSG_OP_SCALE: op_scale<R>(tile, tbits, m); break;
            default: break;
        }
    }
    __syncthreads();
}

// One fused pass over every tile of every member. Tiles are visited grid-stride; each CTA
// handles one tile at a time (CTAs co-resident on an SM overlap each other's copies).
template <typename R>
__global__ void __launch_bounds__(256) k_tile_pass(Cx<R>* __restrict__ state, int64_t member_elems,
                                                   const PassDesc* __restrict__ pass_g,
                                                   const TileOp* __restrict__ ops,
                                                   const Cx<R>* __restrict__ data, int64_t tiles_per_member,
                                                   int64_t total_tiles, int* status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ PassDesc pd;
    Cx<R>* tile = reinterpret_cast<Cx<R>*>(smem_raw);
    if (threadIdx.x == 0) pd = *pass_g;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int K = pd.K, L = pd.L;
    const int nchunks = 1 << (K - L);
    const uint32_t chunk_bytes = (uint32_t)(sizeof(Cx<R>) << L);
    const bool use_bulk = (chunk_bytes % 16) == 0;
    uint32_t parity = 0;
    for (int64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        const int64_t member = t / tiles_per_member;
        const uint64_t tt = (uint64_t)(t - member * tiles_per_member);
        Cx<R>* mem = state + member * member_elems;
        const uint64_t base = deposit(tt, pd.outer, pd.nouter);
        // ---- load
        if (use_bulk) {
            if (threadIdx.x < 32) {
                if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, chunk_bytes * (uint32_t)nchunks);
                __syncwarp();
                for (int c = threadIdx.x; c < nchunks; c += 32)
                    bulk_g2s(tile + ((size_t)c << L), mem + (base | deposit((uint64_t)c, pd.hi, K - L)), chunk_bytes,
                             &bar);
            }
            const bool ok = mbar_wait_bounded(&bar, parity, status);
            if (__syncthreads_or(!ok)) return;  // every thread leaves together on a timeout
            parity ^= 1;
        } else {
            const int n = 1 << K;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                uint64_t g = base | deposit((uint64_t)(i >> L), pd.hi, K - L) | (uint64_t)(i & ((1 << L) - 1));
                tile[i] = mem[g];
            }
        }
        // ---- compute
        run_ops<R>(tile, K, ops + pd.first_op, pd.nops, data, member);
        // ---- store
        if (use_bulk) {
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x < 32) {
                for (int c = threadIdx.x; c < nchunks; c += 32)
                    bulk_s2g(mem + (base | deposit((uint64_t)c, pd.hi, K - L)), tile + ((size_t)c << L), chunk_bytes);
                bulk_commit();
                bulk_wait_read();
            }
            __syncthreads();
        } else {
            const int n = 1 << K;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                uint64_t g = base | deposit((uint64_t)(i >> L), pd.hi, K - L) | (uint64_t)(i & ((1 << L) - 1));
                mem[g] = tile[i];
            }
            __syncthreads();
        }
    }
    if (use_bulk && threadIdx.x < 32) bulk_wait_all();
}

// ------------------------------------------------------------------------ planner

struct Plan {
    std::vector<PassDesc> passes;
    std::vector<TileOp> ops;
};

static int op_bits_ok(const lsg_op& op, int nbits) {
    if (op.kind == LSG_OP_SCALE) return op.nbits == 0;
    if (op.nbits < 1 || op.nbits > LSG_MAX_OP_BITS) return 0;
    if (op.kind == LSG_OP_MATRIX || op.kind == LSG_OP_PERM) {
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

// Greedy fusion: sweep the remaining operators; an operator joins the current pass when its bits
// fit the tile and no operator deferred earlier in the sweep shares a bit with it (so program
// order is kept wherever it matters). Deferred operators start the next sweep.
static Plan plan_passes(const lsg_op* ops, int nops, int nbits, int K, int L) {
    Plan plan;
    std::vector<int> remaining(nops);
    for (int i = 0; i < nops; ++i) remaining[i] = i;
    const uint64_t low = (L >= 64) ? ~0ull : ((1ull << L) - 1);
    while (!remaining.empty()) {
        uint64_t tile = low;
        uint64_t blocked = 0;
        std::vector<int> taken, deferred;
        for (int idx : remaining) {
            const lsg_op& op = ops[idx];
            uint64_t mask = 0;
            for (int i = 0; i < op.nbits; ++i) mask |= 1ull << op.bits[i];
            if (mask & blocked) {
                deferred.push_back(idx);
                blocked |= mask;
                continue;
            }
            uint64_t grown = tile | mask;
            if (__builtin_popcountll(grown) <= K) {
                tile = grown;
                taken.push_back(idx);
            } else {
                deferred.push_back(idx);
                blocked |= mask;
            }
        }
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
            plan.ops.push_back(t);
        }
        plan.passes.push_back(pd);
        remaining.swap(deferred);
    }
    return plan;
}

int tile_bits_for(const lsg_state_s* s) {
    int K = s->precision == LSG_C128 ? 10 : 11;
    if (const char* env = getenv("LSG_TILE_BITS")) K = atoi(env);
    return std::max(0, std::min(K, s->nbits));
}

// Register bits every tile keeps: 2^L contiguous amplitudes = 512 bytes per copy.
int low_bits_for(const lsg_state_s* s) {
    int L = s->precision == LSG_C128 ? 5 : 6;
    if (const char* env = getenv("LSG_LOW_BITS")) L = atoi(env);
    return std::max(0, std::min(L, s->nbits));
}

template <typename R>
static int launch_passes(lsg_state_s* s, const Plan& plan, const void* pool_dev) {
    const int K = plan.passes.empty() ? 0 : plan.passes[0].K;
    const size_t smem = sizeof(Cx<R>) << K;
    auto kern = k_tile_pass<R>;
    if (smem > 48 * 1024) LSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t tiles_per_member = 1ll << (s->nbits - K);
    const int64_t total = tiles_per_member * s->batch;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
    int64_t grid = std::max<int64_t>(1, std::min<int64_t>(total, (int64_t)sms * std::max(per_sm, 1) * 4));
    int* status = device_status();
    if (!status) return fail(LSG_E_CUDA, "cannot allocate the device status word");
    const PassDesc* pd_dev = reinterpret_cast<const PassDesc*>(s->program.ptr);
    const TileOp* ops_dev = reinterpret_cast<const TileOp*>(pd_dev + plan.passes.size());
    for (size_t p = 0; p < plan.passes.size(); ++p) {
        kern<<<(unsigned)grid, 256, smem, s->stream>>>(reinterpret_cast<Cx<R>*>(s->data), s->elems, pd_dev + p,
                                                        ops_dev, reinterpret_cast<const Cx<R>*>(pool_dev),
                                                        tiles_per_member, total, status);
    }
    LSG_CUDA(cudaGetLastError());
    return LSG_OK;
}

int apply_ops(lsg_state_s* s, const lsg_op* ops, int32_t nops, const double* pool, int64_t pool_entries) {
    if (nops < 0 || (nops > 0 && !ops) || pool_entries < 0 || (pool_entries > 0 && !pool))
        return fail(LSG_E_ARG, "lsg_apply: bad operator list or pool");
    for (int i = 0; i < nops; ++i) {
        const lsg_op& op = ops[i];
        if (!op_bits_ok(op, s->nbits)) return fail(LSG_E_ARG, "lsg_apply: operator %d has bad kind or bits", i);
        int64_t need = 1;
        const int64_t d = 1ll << (op.kind == LSG_OP_DEPOL ? 0 : op.nbits);
        if (op.kind == LSG_OP_MATRIX) need = d * d;
        else if (op.kind == LSG_OP_DIAG) need = d;
        else if (op.kind == LSG_OP_PERM) need = 2 * d;
        int64_t last = op.data + need + (s->batch - 1) * op.batch_stride;
        if (op.data < 0 || op.batch_stride < 0 || last > pool_entries)
            return fail(LSG_E_ARG, "lsg_apply: operator %d reads outside the pool", i);
        if (op.kind == LSG_OP_PERM) {
            for (int64_t b = 0; b < s->batch; ++b)
                for (int64_t r = 0; r < d; ++r) {
                    double srcv = pool[2 * (op.data + b * op.batch_stride + d + r)];
                    if (!(srcv >= 0 && srcv < (double)d) || srcv != (double)(int64_t)srcv)
                        return fail(LSG_E_ARG, "lsg_apply: operator %d has a bad permutation", i);
                }
        }
    }
    if (nops == 0) return LSG_OK;
    const int K = tile_bits_for(s);
    const int L = std::min(K, low_bits_for(s));
    Plan plan = plan_passes(ops, nops, s->nbits, K, L);
    if (plan.passes.empty())
        return fail(LSG_E_ARG, "lsg_apply: an operator does not fit a tile of %d bits (%d kept low)", K, L);
    // upload: pass descriptors, tile ops, then the pool in the register's precision
    const size_t head = plan.passes.size() * sizeof(PassDesc) + plan.ops.size() * sizeof(TileOp);
    const size_t head_aligned = (head + 255) & ~size_t(255);
    const size_t elt = s->precision == LSG_C128 ? 16 : 8;
    const size_t total = head_aligned + (size_t)pool_entries * elt;
    std::vector<unsigned char> blob(total);
    std::memcpy(blob.data(), plan.passes.data(), plan.passes.size() * sizeof(PassDesc));
    std::memcpy(blob.data() + plan.passes.size() * sizeof(PassDesc), plan.ops.data(),
                plan.ops.size() * sizeof(TileOp));
    if (s->precision == LSG_C128) {
        std::memcpy(blob.data() + head_aligned, pool, (size_t)pool_entries * 16);
    } else {
        float* f = reinterpret_cast<float*>(blob.data() + head_aligned);
        for (int64_t i = 0; i < 2 * pool_entries; ++i) f[i] = (float)pool[i];
    }
    LSG_CHECK(ensure(s->program, total));
    LSG_CUDA(cudaMemcpyAsync(s->program.ptr, blob.data(), total, cudaMemcpyHostToDevice, s->stream));
    const void* pool_dev = static_cast<unsigned char*>(s->program.ptr) + head_aligned;
    int rc = s->precision == LSG_C128 ? launch_passes<double>(s, plan, pool_dev)
                                      : launch_passes<float>(s, plan, pool_dev);
    LSG_CHECK(rc);
    // the host blob is released on return: make sure the copy has consumed it
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return check_device_status(s->stream);
}

// ------------------------------------------------------------------------ register kernels

template <typename R>
__global__ void k_set_basis(Cx<R>* state, int64_t elems, int64_t batch, int64_t index) {
    const int64_t n = elems * batch;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = i % elems;
        state[i] = Cx<R>(j == index ? R(1) : R(0), R(0));
    }
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
    return LSG_OK;
}

int lsg_max_bits(void) { return kMaxBits; }

int lsg_state_create(int nbits, int precision, int64_t batch, lsg_state* out) {
    clear_error();
    if (!out) return fail(LSG_E_ARG, "lsg_state_create: null output");
    *out = nullptr;
    if (nbits < 0) return fail(LSG_E_ARG, "lsg_state_create: negative bit count");
    if (nbits > kMaxBits) return fail(LSG_E_CAPACITY, "a register of %d bits exceeds the engine's %d", nbits, kMaxBits);
    if (precision != LSG_C128 && precision != LSG_C64) return fail(LSG_E_ARG, "unknown precision %d", precision);
    if (batch < 1) return fail(LSG_E_ARG, "lsg_state_create: batch must be at least 1");
    auto* s = new lsg_state_s();
    s->nbits = nbits;
    s->precision = precision;
    s->batch = batch;
    s->elems = 1ll << nbits;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail(LSG_E_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(e));
    }
    e = cudaMalloc(&s->data, s->member_bytes() * (size_t)batch);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s->stream);
        delete s;
        cudaGetLastError();
        return fail(LSG_E_MEMORY, "cannot allocate %lld bytes of device memory for the register",
                    (long long)(s->member_bytes() * (size_t)batch));
    }
    *out = s;
    return lsg_state_set_basis(s, 0);
}

int lsg_state_free(lsg_state s) {
    clear_error();
    if (!s) return LSG_OK;
    cudaStreamSynchronize(s->stream);
    cudaFree(s->data);
    release(s->program);
    release(s->scratch);
    release(s->scratch2);
    cudaStreamDestroy(s->stream);
    delete s;
    return LSG_OK;
}

int lsg_state_set_basis(lsg_state s, int64_t index) {
    clear_error();
    if (!s) return fail(LSG_E_ARG, "null register");
    if (index < 0 || index >= s->elems) return fail(LSG_E_ARG, "basis index %lld out of range", (long long)index);
    const int64_t n = s->elems * s->batch;
    if (s->precision == LSG_C128)
        k_set_basis<double><<<grid_for(n), 256, 0, s->stream>>>((Cx<double>*)s->data, s->elems, s->batch, index);
    else
        k_set_basis<float><<<grid_for(n), 256, 0, s->stream>>>((Cx<float>*)s->data, s->elems, s->batch, index);
    LSG_CUDA(cudaGetLastError());
    LSG_CUDA(cudaStreamSynchronize(s->stream));
    return LSG_OK;
}

int lsg_state_upload(lsg_state s, const double* host, int64_t nbytes) {
    clear_error();
    if (!s || !host) return fail(LSG_E_ARG, "null argument");
    const int64_t n = s->elems * s->batch;
    if (nbytes != n * 16) return fail(LSG_E_ARG, "upload expects %lld bytes, got %lld", (long long)(n * 16), (long long)nbytes);
    if (s->precision == LSG_C128) {
        LSG_CUDA(cudaMemcpyAsync(s->data, host, (size_t)nbytes, cudaMemcpyHostToDevice, s->stream));
    } else {
        LSG_CHECK(ensure(s->scratch2, (size_t)nbytes));
        LSG_CUDA(cudaMemcpyAsync(s->scratch2.ptr, host, (size_t)nbytes, cudaMemcpyHostToDevice, s->stream));
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
    if (nbytes != n * 16) return fail(LSG_E_ARG, "download expects %lld bytes, got %lld", (long long)(n * 16), (long long)nbytes);
    if (s->precision == LSG_C128) {
        LSG_CUDA(cudaMemcpyAsync(host, s->data, (size_t)nbytes, cudaMemcpyDeviceToHost, s->stream));
    } else {
        LSG_CHECK(ensure(s->scratch2, (size_t)nbytes));
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

}  // extern "C"

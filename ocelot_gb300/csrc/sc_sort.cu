// Deterministic NGP charge deposit: stable radix sort of cell keys followed
// by a segmented sum in particle order.
//
// The reference deposits with np.bincount(inds, Q) (ocelot/cpbd/sc.py:193),
// which adds the charges of each cell sequentially in particle order.  Here
// the keys are sorted by a stable least-significant-digit radix sort (8-bit
// digits, so ceil(key_bits/8) passes), which puts the particles of each cell
// in a contiguous run in particle order; each run is then summed
// sequentially by one thread.  In FP64 this reproduces bincount's sums bit
// for bit; in FP32 the run sum is Kahan-compensated.  The result does not
// depend on scheduling, so it is the same alone and in a batch.
//
// Each radix pass is three launches with no inter-block waiting:
//   hist     per-block digit histogram of a 4096-key tile -> hist[digit][block]
//   rowscan  one warp per digit: exclusive scan along the blocks, digit totals
//   scatter  per block: digit bases from the totals, then 16 rounds of 256 keys,
//            ranking equal digits within a warp by __match_any_sync and across
//            warps by a per-digit prefix in shared memory (stable order:
//            round, warp, lane = particle order)
#include "sc_common.cuh"

namespace ocsc {

constexpr int RT = 256;
constexpr int RITEMS = 16;
constexpr int RTILE = RT * RITEMS;
constexpr int RWARPS = RT / 32;
constexpr unsigned FULLM = 0xffffffffu;

__global__ void __launch_bounds__(RT) k_rhist(const uint32_t* __restrict__ keys, int64_t n, int shift, int bins,
                                              uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RTILE;
    const uint32_t mask = (uint32_t)bins - 1;
#pragma unroll 4
    for (int it = 0; it < RITEMS; ++it) {
        const int64_t i = base + it * RT + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    if (threadIdx.x < bins) hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_rrowscan(uint32_t* __restrict__ hist, int nblk, int bins, uint32_t* __restrict__ tot) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= bins) return;
    uint32_t* row = hist + (size_t)warp * nblk;
    uint32_t carry = 0;
    for (int b0 = 0; b0 < nblk; b0 += 32) {
        const int b = b0 + lane;
        const uint32_t v = b < nblk ? row[b] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULLM, incl, o);
            if (lane >= o) incl += t;
        }
        if (b < nblk) row[b] = carry + incl - v;
        carry += __shfl_sync(FULLM, incl, 31);
    }
    if (lane == 0) tot[warp] = carry;
}

__global__ void __launch_bounds__(RT) k_rscatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                 int64_t n, int shift, int bins, const uint32_t* __restrict__ hist,
                                                 const uint32_t* __restrict__ tot, uint32_t* __restrict__ kout,
                                                 uint32_t* __restrict__ vout) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wsum[RWARPS];
    __shared__ uint32_t wc[RWARPS][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // exclusive scan of the digit totals -> global start of each digit
    const uint32_t tv = tid < bins ? tot[tid] : 0u;
    uint32_t incl = tv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULLM, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t woff = 0;
    for (int w = 0; w < warp; ++w) woff += wsum[w];
    base[tid] = woff + incl - tv + (tid < bins ? hist[(size_t)tid * gridDim.x + blockIdx.x] : 0u);
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t mask = (uint32_t)bins - 1;
    const int64_t tile = (int64_t)blockIdx.x * RTILE;
    for (int r = 0; r < RITEMS; ++r) {
        const int64_t i = tile + (int64_t)r * RT + tid;
        const bool valid = i < n;
        const uint32_t key = valid ? kin[i] : 0u;
        const uint32_t val = valid ? (vin ? vin[i] : (uint32_t)i) : 0u;
        const uint32_t d = valid ? ((key >> shift) & mask) : 256u;
#pragma unroll
        for (int w = 0; w < RWARPS; ++w) wc[w][tid] = 0u;
        __syncthreads();
        const uint32_t peers = __match_any_sync(FULLM, d);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wc[warp][d] = __popc(peers);
        __syncthreads();
        if (tid < bins) {
            uint32_t run = base[tid];
#pragma unroll
            for (int w = 0; w < RWARPS; ++w) {
                const uint32_t c = wc[w][tid];
                wc[w][tid] = run;
                run += c;
            }
            base[tid] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wc[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

static int sort_blocks(int64_t n) { return (int)((n + RTILE - 1) / RTILE); }

size_t sort_scratch_bytes(int64_t n, int key_bits) {
    (void)key_bits;
    const size_t nb = (size_t)(sort_blocks(n) > 0 ? sort_blocks(n) : 1);
    return align_up(4 * (size_t)n) * 2 + align_up(256 * nb * 4) + align_up(256 * 4);
}

cudaError_t launch_sort(const uint32_t* keys_in, int64_t n, int key_bits, uint32_t* keys_out, uint32_t* perm_out,
                        uint32_t* tmp_k, uint32_t* tmp_v, uint32_t* hist, uint32_t* tot, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int nb = sort_blocks(n);
    const int passes = key_bits <= 0 ? 1 : (key_bits + 7) / 8;
    const uint32_t* sk = keys_in;
    const uint32_t* sv = nullptr;
    bool to_out = (passes % 2) == 1;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        int dbits = key_bits - shift;
        dbits = dbits > 8 ? 8 : (dbits < 1 ? 1 : dbits);
        const int bins = 1 << dbits;
        uint32_t* dk = to_out ? keys_out : tmp_k;
        uint32_t* dv = to_out ? perm_out : tmp_v;
        k_rhist<<<nb, RT, 0, s>>>(sk, n, shift, bins, hist);
        k_rrowscan<<<(bins * 32 + 255) / 256, 256, 0, s>>>(hist, nb, bins, tot);
        k_rscatter<<<nb, RT, 0, s>>>(sk, sv, n, shift, bins, hist, tot, dk, dv);
        sk = dk;
        sv = dv;
        to_out = !to_out;
    }
    return cudaGetLastError();
}

// one thread per run of equal keys sums the run in particle order
template <typename R>
__global__ void k_deposit(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ perm,
                          const double* __restrict__ q, int64_t n, R* __restrict__ qgrid, const ScState* st) {
    if (st->status) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t key = sk[j];
        if (j > 0 && sk[j - 1] == key) continue;
        if (sizeof(R) == 8) {
            double sum = 0.0;
            for (int64_t m = j; m < n && sk[m] == key; ++m) sum = __dadd_rn(sum, q[perm[m]]);
            qgrid[key] = (R)sum;
        } else {
            float sum = 0.f, comp = 0.f;
            for (int64_t m = j; m < n && sk[m] == key; ++m) {
                const float y = __fsub_rn((float)q[perm[m]], comp);
                const float t = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(t, sum), y);
                sum = t;
            }
            qgrid[key] = (R)sum;
        }
    }
}

cudaError_t launch_deposit(const Plan& p, const Layout& L, char* ws, const double* q, int64_t n, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const size_t ncell = (size_t)p.nx * p.ny * p.nz;
    const size_t rs = p.prec == SC_FP64 ? 8 : 4;
    cudaError_t e = cudaMemsetAsync(ws + L.qgrid, 0, ncell * rs, s);
    if (e) return e;
    int64_t b = (n + 255) / 256;
    if (b > p.part_blocks) b = p.part_blocks;
    if (b < 1) b = 1;
    const uint32_t* sk = reinterpret_cast<const uint32_t*>(ws + L.sort_keys);
    const uint32_t* pm = reinterpret_cast<const uint32_t*>(ws + L.sort_perm);
    if (p.prec == SC_FP64)
        k_deposit<double><<<(int)b, 256, 0, s>>>(sk, pm, q, n, reinterpret_cast<double*>(ws + L.qgrid), st);
    else
        k_deposit<float><<<(int)b, 256, 0, s>>>(sk, pm, q, n, reinterpret_cast<float*>(ws + L.qgrid), st);
    return cudaGetLastError();
}

}  // namespace ocsc

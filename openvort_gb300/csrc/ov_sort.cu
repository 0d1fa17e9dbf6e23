// ov_sort.cu - radix sort of the octree path keys and a device-wide scan.
//
// Keys are 64-bit (member id, out-of-box bit, cell path; EMPTY slots all
// ones); the payload is the node id.  An LSD radix sort with 8-bit digits runs over the upper
// 32 bits (4 passes: 10 octree levels and one bit); nodes that still share
// those bits (the same level-10 cell) are then put in full-key order by an
// insertion sort per run.  LSD passes are stable, so input (node id) order
// breaks ties and the result is deterministic.
//
// Each pass is three kernels: per-tile digit histogram, scan of the
// (digit, tile) table, stable scatter.  HBM traffic per pass: read 12 B and
// write 12 B per slot.
#include "ov_internal.cuh"

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                       // items per thread
constexpr int kTile = kSortThreads * kSortItems;     // 4096 slots per block
constexpr int kWarps = kSortThreads / 32;

__global__ void rs_hist(const uint64_t *__restrict__ keys, int n, int shift, int ntiles,
                        int *__restrict__ hist)
{
    __shared__ int h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int base = blockIdx.x * kTile;
    for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
        int g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 0xFF], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * ntiles + blockIdx.x] = h[d];
}

// Exclusive scan of the digit-major table hist[256*ntiles] in one block
// (small tables: one launch instead of the device-wide scan's three).
__global__ void rs_scan(int *__restrict__ hist, int total)
{
    __shared__ int part[1024];
    int per = (total + blockDim.x - 1) / blockDim.x;
    int b = threadIdx.x * per, e = min(total, b + per);
    int s = 0;
    for (int i = b; i < e; ++i) s += hist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - s;
    for (int i = b; i < e; ++i) {
        int v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// Stable scatter: items of a tile are ordered (warp, round, lane); each warp
// counts digits with match_any, the per-warp counts are scanned across warps
// and a running per-(warp,digit) counter hands out ranks.
__global__ void rs_scatter(const uint64_t *__restrict__ kin, const int *__restrict__ vin,
                           uint64_t *__restrict__ kout, int *__restrict__ vout, int n, int shift,
                           int ntiles, const int *__restrict__ hist)
{
    __shared__ int wc[kWarps][256];
    __shared__ int gbase[256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kWarps * 256; i += blockDim.x) (&wc[0][0])[i] = 0;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) gbase[d] = hist[d * ntiles + blockIdx.x];
    __syncthreads();
    const int wbase = blockIdx.x * kTile + warp * (kSortItems * 32);
    uint64_t k[kSortItems];
    int v[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int g = wbase + r * 32 + lane;
        k[r] = g < n ? kin[g] : 0;
        v[r] = g < n ? vin[g] : 0;
    }
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int g = wbase + r * 32 + lane;
        unsigned act = __ballot_sync(0xffffffffu, g < n);
        if (g < n) {
            int d = (int)((k[r] >> shift) & 0xFF);
            unsigned m = __match_any_sync(act, d);
            if ((m & lt) == 0) wc[warp][d] += __popc(m);
        }
        __syncwarp();
    }
    __syncthreads();
    // exclusive scan over warps per digit
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        int run = 0;
        for (int w = 0; w < kWarps; ++w) {
            int c = wc[w][d];
            wc[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int g = wbase + r * 32 + lane;
        unsigned act = __ballot_sync(0xffffffffu, g < n);
        if (g < n) {
            int d = (int)((k[r] >> shift) & 0xFF);
            unsigned m = __match_any_sync(act, d);
            int base = wc[warp][d];
            int pos = gbase[d] + base + __popc(m & lt);
            kout[pos] = k[r];
            vout[pos] = v[r];
            __syncwarp(m);
            if ((m & lt) == 0) wc[warp][d] = base + __popc(m);
        }
        __syncwarp();
    }
}

// Order each run of equal upper-32-bit keys by the full key (insertion
// sort, stable): in-box and out-of-box keys of every member.  Only EMPTY
// slots have all-ones upper bits (the key layout keeps every other key
// below: member ids are never all ones, out-of-box keys keep the bit under
// the out-of-box bit clear); their run stays in id order.
__global__ void rs_fixup(uint64_t *__restrict__ keys, int *__restrict__ vals, int n, int *counters)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t hi = (uint32_t)(keys[i] >> 32);
    if (hi == 0xFFFFFFFFu) return;
    if (i > 0 && (uint32_t)(keys[i - 1] >> 32) == hi) return;
    int e = i + 1;
    while (e < n && (uint32_t)(keys[e] >> 32) == hi) ++e;
    if (e - i == 1) return;
    atomicMax(&counters[TC_MAXRUN], e - i);
    for (int a = i + 1; a < e; ++a) {
        uint64_t kk = keys[a];
        int vv = vals[a];
        int b = a - 1;
        while (b >= i && keys[b] > kk) {
            keys[b + 1] = keys[b];
            vals[b + 1] = vals[b];
            --b;
        }
        keys[b + 1] = kk;
        vals[b + 1] = vv;
    }
}

// ---------------------------------------------------------------- scan
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    int warp_off = warp > 0 ? sh[warp - 1] : 0;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

__global__ void scan_tiles(const int *__restrict__ in, int *__restrict__ out, int n_max,
                           const int *n_dev, int *__restrict__ tile_sums)
{
    __shared__ int sh[32];
    int n = n_dev ? min(*n_dev, n_max) : n_max;
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        s += v[i];
    }
    int total;
    int off = block_excl_scan(s, sh, total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i <= n_max) out[base + i] = off;
        off += v[i];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void scan_sums(int *__restrict__ tile_sums, int ntiles)
{
    __shared__ int sh[32];
    int run = 0;
    for (int b = 0; b < ntiles; b += blockDim.x) {
        int i = b + threadIdx.x;
        int v = i < ntiles ? tile_sums[i] : 0;
        int total;
        int off = block_excl_scan(v, sh, total);
        if (i < ntiles) tile_sums[i] = run + off;
        run += total;
    }
}

__global__ void scan_add(int *__restrict__ out, int n_max, const int *n_dev, const int *__restrict__ tile_sums,
                         int add)
{
    int n = n_dev ? min(*n_dev, n_max) : n_max;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    out[i] += tile_sums[i / kScanTile] + add;
}

}  // namespace

void ov_scan_exclusive(ov_ctx *c, const int *in, int *out, int n_max, const int *n_dev, int add, int *tmp,
                       cudaStream_t s);

// Radix sort of t.keys / t.order (n slots); the digit tables of more than
// 32 tiles are scanned in place by the device-wide scan (the table has room
// for its total).
void ov_sort_keys(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s)
{
    if (n <= 0) return;
    int ntiles = (n + kTile - 1) / kTile;
    uint64_t *ka = t.keys, *kb = t.keys_alt;
    int *va = t.order, *vb = t.order_alt;
    for (int pass = 0; pass < 4; ++pass) {
        int shift = 32 + 8 * pass;
        rs_hist<<<ntiles, kSortThreads, 0, s>>>(ka, n, shift, ntiles, t.sort_hist);
        if (ntiles <= 32) {
            rs_scan<<<1, 1024, 0, s>>>(t.sort_hist, 256 * ntiles);
            c->launches += 1;
        } else {
            ov_scan_exclusive(c, t.sort_hist, t.sort_hist, 256 * ntiles, nullptr, 0, t.scan_tmp, s);
        }
        rs_scatter<<<ntiles, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift, ntiles, t.sort_hist);
        c->launches += 2;
        uint64_t *tk = ka; ka = kb; kb = tk;
        int *tv = va; va = vb; vb = tv;
    }
    // after 4 passes the result is back in t.keys / t.order
    rs_fixup<<<(n + 255) / 256, 256, 0, s>>>(ka, va, n, t.counters);
    c->launches += 1;
}

int ov_sort_hist_ints(int cap) { return 256 * ((cap + kTile - 1) / kTile) + 256; }

// out[i] = add + sum(in[0..i)) for i in [0, n], n = min(*n_dev, n_max).
void ov_scan_exclusive(ov_ctx *c, const int *in, int *out, int n_max, const int *n_dev, int add,
                       int *tmp, cudaStream_t s)
{
    int ntiles = (n_max + 1 + kScanTile - 1) / kScanTile;
    scan_tiles<<<ntiles, kScanThreads, 0, s>>>(in, out, n_max, n_dev, tmp);
    scan_sums<<<1, 1024, 0, s>>>(tmp, ntiles);
    scan_add<<<(n_max + 1 + 255) / 256, 256, 0, s>>>(out, n_max, n_dev, tmp, add);
    c->launches += 3;
}

int ov_scan_tmp_ints(int n_max) { return (n_max + 1 + kScanTile - 1) / kScanTile + 32; }

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
constexpr int kWarps = kSortThreads / 32;
// Items per thread: 16 (4096-slot tiles), or 4 (1024-slot tiles) when the
// slots are few enough that 4096-slot tiles would leave most SMs idle.
constexpr int kItemsLarge = 16, kItemsSmall = 4;
constexpr int kSmallSortSlots = 1 << 19;
__host__ __device__ constexpr int sort_tile(int items) { return kSortThreads * items; }

// Exclusive scan of one int per thread over the block (blockDim a multiple
// of 32, at most 1024); total gets the block's sum.
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

// Per-tile histogram of the pass's digit (digit-major table hist[d * ntiles
// + tile]); with tot, also the totals of all four digits over every key,
// which the later passes' digit offsets start from (the keys of a pass are
// a permutation of the first pass's).  Same-digit lanes of a warp add once.
template <int kSortItems>
__global__ void rs_hist(const uint64_t *__restrict__ keys, int n, int shift, int ntiles,
                        int *__restrict__ hist, int *__restrict__ tot)
{
    constexpr int kTile = sort_tile(kSortItems);
    __shared__ int h[4][256];
    const int np = tot ? 4 : 1;
    for (int i = threadIdx.x; i < np * 256; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
    uint64_t k[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int g = base + r * kSortThreads + threadIdx.x;
        k[r] = g < n ? keys[g] : 0;
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int g = base + r * kSortThreads + threadIdx.x;
        const unsigned act = __ballot_sync(0xffffffffu, g < n);
        if (g < n) {
            for (int p = 0; p < np; ++p) {
                const int sh = tot ? 32 + 8 * p : shift;
                const int d = (int)((k[r] >> sh) & 0xFF);
                const unsigned m = __match_any_sync(act, d);
                if (lane == __ffs(m) - 1) atomicAdd(&h[p][d], __popc(m));
            }
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * ntiles + blockIdx.x] = h[tot ? (shift - 32) / 8 : 0][d];
    if (tot)
        for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
            if ((&h[0][0])[i]) atomicAdd(&tot[i], (&h[0][0])[i]);
}

// Digit offsets of a pass: block d turns row d of the table into global
// output offsets, the keys of smaller digits (from the totals) plus the
// row's prefix over tiles.
__global__ void rs_rowscan(int *__restrict__ hist, int ntiles, const int *__restrict__ tot)
{
    __shared__ int sh[32];
    const int d = blockIdx.x;
    int total;
    block_excl_scan(threadIdx.x < d ? tot[threadIdx.x] : 0, sh, total);
    int run = total;
    int *row = hist + (size_t)d * ntiles;
    for (int b = 0; b < ntiles; b += blockDim.x) {
        const int i = b + threadIdx.x;
        const int v = i < ntiles ? row[i] : 0;
        const int off = block_excl_scan(v, sh, total);
        if (i < ntiles) row[i] = run + off;
        run += total;
    }
}

// Stable scatter: items of a tile are ordered (warp, round, lane); each warp
// counts digits with match_any, the per-warp counts are scanned across warps
// and a running per-(warp,digit) counter hands out ranks.  The tile is put in
// digit order in shared memory first, so that each digit's run is written
// out by consecutive threads (keys, then the ids through the same buffer).
template <int kSortItems>
__global__ void rs_scatter(const uint64_t *__restrict__ kin, const int *__restrict__ vin,
                           uint64_t *__restrict__ kout, int *__restrict__ vout, int n, int shift,
                           int ntiles, const int *__restrict__ hist)
{
    constexpr int kTile = sort_tile(kSortItems);
    __shared__ uint64_t sk[kTile];        // the tile in digit order (keys, then ids)
    __shared__ uint8_t sd[kTile];         // digit of each staged slot
    __shared__ int wc[kWarps][256];
    __shared__ int gbase[256], boff[256];
    __shared__ int sh[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kWarps * 256; i += blockDim.x) (&wc[0][0])[i] = 0;
    // (hist null: the keys are one tile, and a digit's output offset is its
    // start in the tile)
    for (int d = threadIdx.x; d < 256; d += blockDim.x) gbase[d] = hist ? hist[d * ntiles + blockIdx.x] : 0;
    __syncthreads();
    const int tbase = blockIdx.x * kTile;
    const int tn = min(kTile, n - tbase);
    const int wbase = tbase + warp * (kSortItems * 32);
    uint64_t k[kSortItems];
    int v[kSortItems], lp[kSortItems];
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
    // exclusive scan over warps per digit; the tile's digit totals scanned
    // over digits give each digit's start in the staged tile
    int dig_total = 0;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        int run = 0;
        for (int w = 0; w < kWarps; ++w) {
            int c = wc[w][d];
            wc[w][d] = run;
            run += c;
        }
        dig_total = run;
    }
    {
        int tot_all;
        const int off = block_excl_scan(threadIdx.x < 256 ? dig_total : 0, sh, tot_all);
        if (threadIdx.x < 256) {
            boff[threadIdx.x] = off;
            if (!hist) gbase[threadIdx.x] = off;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int g = wbase + r * 32 + lane;
        unsigned act = __ballot_sync(0xffffffffu, g < n);
        lp[r] = -1;
        if (g < n) {
            int d = (int)((k[r] >> shift) & 0xFF);
            unsigned m = __match_any_sync(act, d);
            int base = wc[warp][d];
            lp[r] = boff[d] + base + __popc(m & lt);
            sk[lp[r]] = k[r];
            sd[lp[r]] = (uint8_t)d;
            __syncwarp(m);
            if ((m & lt) == 0) wc[warp][d] = base + __popc(m);
        }
        __syncwarp();
    }
    __syncthreads();
    for (int j = threadIdx.x; j < tn; j += blockDim.x) {
        const int d = sd[j];
        kout[gbase[d] + j - boff[d]] = sk[j];
    }
    __syncthreads();
    int *sv = reinterpret_cast<int *>(sk);
#pragma unroll
    for (int r = 0; r < kSortItems; ++r)
        if (lp[r] >= 0) sv[lp[r]] = v[r];
    __syncthreads();
    for (int j = threadIdx.x; j < tn; j += blockDim.x) {
        const int d = sd[j];
        vout[gbase[d] + j - boff[d]] = sv[j];
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

// Radix sort of t.keys / t.order (n slots): per pass a tile histogram, the
// digit offsets (one block per digit) and the scatter; the digit totals of
// all passes come with the first histogram.
template <int kSortItems>
static void sort_passes(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s)
{
    const int ntiles = (n + sort_tile(kSortItems) - 1) / sort_tile(kSortItems);
    uint64_t *ka = t.keys, *kb = t.keys_alt;
    int *va = t.order, *vb = t.order_alt;
    int *tot = t.sort_hist + 256 * (size_t)ntiles;   // 4 x 256 digit totals
    if (ntiles > 1) cudaMemsetAsync(tot, 0, 4 * 256 * sizeof(int), s);
    for (int pass = 0; pass < 4; ++pass) {
        int shift = 32 + 8 * pass;
        if (ntiles > 1) {
            rs_hist<kSortItems><<<ntiles, kSortThreads, 0, s>>>(ka, n, shift, ntiles, t.sort_hist,
                                                               pass == 0 ? tot : nullptr);
            rs_rowscan<<<256, kSortThreads, 0, s>>>(t.sort_hist, ntiles, tot + 256 * pass);
            c->launches += 2;
        }
        // one tile: the scatter's own digit starts are the offsets
        rs_scatter<kSortItems><<<ntiles, kSortThreads, 0, s>>>(ka, va, kb, vb, n, shift, ntiles,
                                                              ntiles > 1 ? t.sort_hist : nullptr);
        c->launches += 1;
        uint64_t *tk = ka; ka = kb; kb = tk;
        int *tv = va; va = vb; vb = tv;
    }
    // after 4 passes the result is back in t.keys / t.order
    rs_fixup<<<(n + 255) / 256, 256, 0, s>>>(ka, va, n, t.counters);
    c->launches += 1;
}

void ov_sort_keys(ov_ctx *c, TreeBuf &t, int n, cudaStream_t s)
{
    if (n <= 0) return;
    // one 4,096-slot tile when the keys fit in it; 1,024-slot tiles up to
    // kSmallSortSlots (more blocks than SMs); 4,096-slot tiles above
    if (n <= sort_tile(kItemsLarge) || n > kSmallSortSlots) sort_passes<kItemsLarge>(c, t, n, s);
    else sort_passes<kItemsSmall>(c, t, n, s);
}

int ov_sort_hist_ints(int cap)
{
    const int tile = cap <= sort_tile(kItemsLarge) || cap > kSmallSortSlots ? sort_tile(kItemsLarge)
                                                                            : sort_tile(kItemsSmall);
    return 256 * ((cap + tile - 1) / tile) + 4 * 256;
}

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

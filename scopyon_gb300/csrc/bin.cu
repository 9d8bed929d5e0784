// Counting sort of splat records by tile.
//
// The reference adds each particle's footprint straight into the image
// (src/scopyon/_epifm.py:1262-1264, :277-282).  Here each record is filed
// under the tile that holds its first footprint pixel, so one CTA can sum all
// of a tile's footprints (which reach into a halo past the tile) in shared
// memory with no global atomics on pixels.  Box-path and summed-area-path
// records go to separate bins (bin t and n_tiles + t for tile t).  Counting a
// record into its bin (one atomic add) also gives its rank in the bin; after
// an exclusive scan of the counts each record is stored at its bin's offset
// plus its rank, and each bin's list is then sorted by record index: the
// final order is the reference's own accumulation order (sub-step, then
// particle) and does not depend on scheduling.  A record producer can do the
// counting itself (sc_bin_record), leaving scan, placement and sort to
// sc_bin_finish.
#include <mutex>

#include "sc_common.cuh"
#include "bin.cuh"

namespace {

// Per-bin counts with global atomics (about 50 records per bin, spread over
// thousands of bins, so contention is low).  With rank, each record's bin and
// rank within the bin are kept for the placement pass.
__global__ void bin_count_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g,
                                 int32_t *tile_count, int32_t *rec_bin, int32_t *rec_rank,
                                 int32_t *status) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rec; r += gridDim.x * blockDim.x) {
        if (sc::record_malformed(recs[r]))
            sc::flag_status(status, 6, r, recs[r].i_start, recs[r].j_start);
        if (rec_bin)
            sc::bin_record(g, recs[r], r, tile_count, rec_bin, rec_rank);
        else {
            const int t = sc::record_tile(recs[r], r, g);
            if (t >= 0) atomicAdd(&tile_count[t], 1);
        }
    }
}

constexpr int kScanThreads = 1024, kScanItems = 8;

__device__ __forceinline__ void load8(const int32_t *p, bool vec, int n_left, int32_t v[8]) {
    if (vec && n_left >= 8) {
        const int4 a = *reinterpret_cast<const int4 *>(p), b = *reinterpret_cast<const int4 *>(p + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = u < n_left ? p[u] : 0;
    }
}

__device__ __forceinline__ void store8(int32_t *p, bool vec, int n_left, const int32_t v[8]) {
    if (vec && n_left >= 8) {
        *reinterpret_cast<int4 *>(p) = make_int4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<int4 *>(p + 4) = make_int4(v[4], v[5], v[6], v[7]);
    } else {
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (u < n_left) p[u] = v[u];
    }
}

// Single-CTA exclusive scan of the bin counts -> tile_start[0..n_bins] (and
// the scatter cursors when given).  Each thread scans 8 consecutive bins, with
// 16-byte loads and stores where the arrays allow.
__global__ void __launch_bounds__(kScanThreads)
bin_tile_scan_kernel(const int32_t *tile_count, int n_bins, int32_t *tile_start, int32_t *cursor) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool vin = ((uintptr_t)tile_count & 15) == 0;
    const bool vout = ((uintptr_t)tile_start & 15) == 0 && (!cursor || ((uintptr_t)cursor & 15) == 0);
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n_bins; base += kScanThreads * kScanItems) {
        const int t0 = base + threadIdx.x * kScanItems;
        const int n_left = n_bins - t0;
        int32_t v[kScanItems], sum = 0;
        load8(tile_count + t0, vin, n_left, v);
#pragma unroll
        for (int u = 0; u < kScanItems; ++u) sum += v[u];
        int32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t n = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += n;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t n = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += n;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        int32_t run = x - sum + (warp > 0 ? warp_tot[warp - 1] : 0) + carry_s;
        int32_t out[kScanItems];
#pragma unroll
        for (int u = 0; u < kScanItems; ++u) {
            out[u] = run;
            run += v[u];
        }
        if (n_left > 0) {
            store8(tile_start + t0, vout, n_left, out);
            if (cursor) store8(cursor + t0, vout, n_left, out);
        }
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry_s = run;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_start[n_bins] = carry_s;
}

// Each record to its bin's offset plus its rank.
__global__ void bin_place_kernel(const int32_t *rec_bin, const int32_t *rec_rank, int n_rec,
                                 const int32_t *tile_start, int32_t *items, int32_t *status) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rec; r += gridDim.x * blockDim.x) {
        const int t = rec_bin[r];
        if (t < 0) continue;
        const int pos = __ldg(tile_start + t) + rec_rank[r];
        if (sc::in_range(pos, n_rec, status, 4)) items[pos] = r;
    }
}

// Without rank storage: one atomic cursor per bin, each record's bin
// recomputed from its head.
__global__ void bin_scatter_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g,
                                   int32_t *cursor, int32_t *items, int32_t *status) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rec; r += gridDim.x * blockDim.x) {
        const int t = sc::record_tile(recs[r], r, g);
        if (t < 0 || !sc::in_range(t, 2 * g.n_tiles, status, 5)) continue;
        const int pos = atomicAdd(&cursor[t], 1);
        if (sc::in_range(pos, n_rec, status, 4)) items[pos] = r;
    }
}

// Bitonic sort of 32 PL values held PL per lane (element e = PL lane + r),
// ascending; padding values sort to the end.
template <int PL>
__device__ __forceinline__ void warp_sort(int32_t v[PL], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * PL; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= PL) {
#pragma unroll
                for (int r = 0; r < PL; ++r) {
                    const int32_t other = __shfl_xor_sync(0xffffffffu, v[r], j / PL);
                    const int e = lane * PL + r;
                    const bool keep_min = ((e & k) == 0) == ((e & j) == 0);
                    v[r] = keep_min ? min(v[r], other) : max(v[r], other);
                }
            } else {
#pragma unroll
                for (int r = 0; r < PL; ++r) {
                    const int q = r ^ j;
                    if (r < q) {
                        const bool up = ((lane * PL + r) & k) == 0;
                        const int32_t a = v[r], b = v[q];
                        if ((a > b) == up) {
                            v[r] = b;
                            v[q] = a;
                        }
                    }
                }
            }
        }
    }
}

template <int PL>
__device__ __forceinline__ void warp_sort_list(int32_t *list, int n, int lane) {
    int32_t v[PL];
#pragma unroll
    for (int r = 0; r < PL; ++r) {
        const int e = lane * PL + r;
        v[r] = e < n ? list[e] : INT32_MAX;
    }
    warp_sort<PL>(v, lane);
#pragma unroll
    for (int r = 0; r < PL; ++r) {
        const int e = lane * PL + r;
        if (e < n) list[e] = v[r];
    }
}

// Ascending compare-exchange of a[i] and a[l] (l > i); positions >= n hold
// +inf implicitly and are never touched.
__device__ __forceinline__ void cmp_swap(int32_t *a, int i, int l, int n) {
    if (l >= n) return;
    const int32_t x = a[i], y = a[l];
    if (x > y) {
        a[i] = y;
        a[l] = x;
    }
}

// Bitonic sorting network in its "flip" form (every comparator ascending), so
// that a list of any length n sorts in place with virtual +inf padding up to
// the next power of two; run by one warp on a list in global memory (bins of
// more than 512 records, which only dense clusters of emitters produce).
__device__ void warp_flip_sort(int32_t *a, int n, int lane) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int k = 2; k <= n2; k <<= 1) {
        for (int i = lane; i < n2; i += 32) {
            const int l = i ^ (k - 1);
            if (l > i) cmp_swap(a, i, l, n);
        }
        __syncwarp();
        for (int j = k >> 2; j > 0; j >>= 1) {
            for (int i = lane; i < n2; i += 32) {
                const int l = i ^ j;
                if (l > i) cmp_swap(a, i, l, n);
            }
            __syncwarp();
        }
    }
}

constexpr int kSortWarps = 8;

// One warp per bin: the bin's record indices sorted ascending, in registers
// up to 512 of them (1, 2, 4, 8 or 16 per lane).  Longer lists go to `big` (a count
// and the bin indices) for bin_sort_big_kernel, or, without that list, are
// sorted here in global memory.
__global__ void __launch_bounds__(kSortWarps * 32)
bin_sort_kernel(const int32_t *tile_start, int n_bins, int32_t *items, int32_t *big) {
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.x * kSortWarps + (threadIdx.x >> 5);
    if (t >= n_bins) return;
    const int b0 = tile_start[t], n = tile_start[t + 1] - b0;
    if (n <= 1) return;
    int32_t *list = items + b0;
    // the smallest register network that holds the list
    if (n <= 32)
        warp_sort_list<1>(list, n, lane);
    else if (n <= 64)
        warp_sort_list<2>(list, n, lane);
    else if (n <= 128)
        warp_sort_list<4>(list, n, lane);
    else if (n <= 256)
        warp_sort_list<8>(list, n, lane);
    else if (n <= 512)
        warp_sort_list<16>(list, n, lane);
    else if (big) {
        if (lane == 0) big[1 + atomicAdd(big, 1)] = t;
    } else {
        warp_flip_sort(list, n, lane);
    }
}

constexpr int kBigThreads = 512;
constexpr int kBigSmem = 12288;  // list entries sorted in shared memory (48 KB)

// Flip-form bitonic network run by a whole CTA on `a` (shared or global).
__device__ void cta_flip_sort(int32_t *a, int n) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int k = 2; k <= n2; k <<= 1) {
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            const int l = i ^ (k - 1);
            if (l > i) cmp_swap(a, i, l, n);
        }
        __syncthreads();
        for (int j = k >> 2; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) cmp_swap(a, i, l, n);
            }
            __syncthreads();
        }
    }
}

// The long lists: CTAs take bins from the list in turn and sort each with the
// whole CTA, in shared memory up to kBigSmem entries.
__global__ void __launch_bounds__(kBigThreads)
bin_sort_big_kernel(const int32_t *tile_start, const int32_t *big, int32_t *items) {
    __shared__ int32_t buf[kBigSmem];
    const int count = big[0];
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int t = big[1 + q];
        const int b0 = tile_start[t], n = tile_start[t + 1] - b0;
        int32_t *list = items + b0;
        if (n <= kBigSmem) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = list[i];
            __syncthreads();
            cta_flip_sort(buf, n);
            for (int i = threadIdx.x; i < n; i += blockDim.x) list[i] = buf[i];
        } else {
            cta_flip_sort(list, n);
        }
        __syncthreads();
    }
}

// Per-bin sort of the placed lists; `big` (count + list, cleared here) takes
// the long ones to a CTA each when the workspace holds it.
int bin_sort(int n_bins, int32_t *tile_start, int32_t *items, int32_t *big, cudaStream_t s) {
    if (big) {
        int rc = sc::cuda_status(cudaMemsetAsync(big, 0, sizeof(int32_t), s), "bin sort");
        if (rc) return rc;
    }
    bin_sort_kernel<<<(n_bins + kSortWarps - 1) / kSortWarps, kSortWarps * 32, 0, s>>>(
        tile_start, n_bins, items, big);
    if (big) bin_sort_big_kernel<<<152 * 2, kBigThreads, 0, s>>>(tile_start, big, items);
    return sc::launch_status("bin sort");
}

// ---------------------------------------------------------------------------
// Large record sets: a stable LSD radix sort of the record indices by bin
// instead of placement by atomic rank plus a sort of every list.  Input is
// rec_bin in record order (bin -1: key n_bins, after every bin); each pass
// partitions by one digit of at most 9 bits and keeps the order of equal
// digits, so the result is ordered by bin and then by record index: the
// same lists as placement plus sort.  A pass is three kernels: per-block
// digit counts (blocks of 2048 records), a scan over blocks per digit, and
// the scatter, where each warp ranks its records among equal digits with
// __match_any_sync in record order.

constexpr int kRxThreads = 512, kRxWarps = kRxThreads / 32, kRxPerWarp = 128;
constexpr int kRxBlock = kRxWarps * kRxPerWarp;  // 2048 records
constexpr int kRxMaxBits = 9, kRxMaxBuckets = 1 << kRxMaxBits;
constexpr int kRxScanThreads = 1024;

__device__ __forceinline__ int rx_key(const int32_t *keys, int q, int sentinel) {
    const int k = keys[q];
    return k < 0 ? sentinel : k;
}

// counts[d * nb + b] = records of block b whose digit is d.
__global__ void __launch_bounds__(kRxThreads)
radix_upsweep_kernel(const int32_t *__restrict__ keys, int n, int sentinel, int shift, int bits,
                     int nb, int32_t *__restrict__ counts) {
    __shared__ int32_t hist[kRxMaxBuckets];
    const int buckets = 1 << bits;
    for (int d = threadIdx.x; d < buckets; d += kRxThreads) hist[d] = 0;
    __syncthreads();
    const int q0 = blockIdx.x * kRxBlock, q1 = min(n, q0 + kRxBlock);
    for (int q = q0 + threadIdx.x; q < q1; q += kRxThreads)
        atomicAdd(&hist[(rx_key(keys, q, sentinel) >> shift) & (buckets - 1)], 1);
    __syncthreads();
    for (int d = threadIdx.x; d < buckets; d += kRxThreads)
        counts[(size_t)d * nb + blockIdx.x] = hist[d];
}

// Inclusive scan over a CTA of kRxScanThreads / kRxThreads threads; returns
// this thread's inclusive value and leaves the CTA total in *total_out.
template <int NT>
__device__ __forceinline__ int cta_inclusive_scan(int v, int32_t *warp_tot, int *total_out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = lane < NT / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int r = x + (warp ? warp_tot[warp - 1] : 0);
    *total_out = warp_tot[NT / 32 - 1];
    __syncthreads();
    return r;
}

// One CTA per digit d: counts[d][0 .. nb) becomes its exclusive scan over
// blocks, total[d] the digit's record count.
__global__ void __launch_bounds__(kRxScanThreads)
radix_scan_kernel(int32_t *__restrict__ counts, int nb, int32_t *__restrict__ total) {
    __shared__ int32_t warp_tot[32];
    int32_t *c = counts + (size_t)blockIdx.x * nb;
    int carry = 0;
    for (int base = 0; base < nb; base += kRxScanThreads) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? c[i] : 0;
        int tot;
        const int incl = cta_inclusive_scan<kRxScanThreads>(v, warp_tot, &tot);
        if (i < nb) c[i] = carry + incl - v;
        carry += tot;
    }
    if (threadIdx.x == 0) total[blockIdx.x] = carry;
}

// Stable scatter of block b: position = start of the digit (scan of the
// totals) + records of the digit in earlier blocks + earlier warps of this
// block + rank within the warp (32 records at a time, in record order).
__global__ void __launch_bounds__(kRxThreads, 3)
radix_downsweep_kernel(const int32_t *__restrict__ keys_in, const int32_t *__restrict__ vals_in,
                       int n, int sentinel, int shift, int bits, int nb,
                       const int32_t *__restrict__ counts, const int32_t *__restrict__ total,
                       int32_t *__restrict__ keys_out, int32_t *__restrict__ vals_out) {
    __shared__ int32_t whist[kRxWarps][kRxMaxBuckets];
    __shared__ int32_t base_s[kRxMaxBuckets];
    __shared__ int32_t warp_tot[32];
    const int buckets = 1 << bits;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    {
        const int d = threadIdx.x;  // buckets <= kRxThreads
        const int v = d < buckets ? total[d] : 0;
        int tot;
        const int incl = cta_inclusive_scan<kRxThreads>(v, warp_tot, &tot);
        if (d < buckets) base_s[d] = incl - v + counts[(size_t)d * nb + blockIdx.x];
    }
    for (int d = lane; d < buckets; d += 32) whist[warp][d] = 0;
    __syncwarp();
    const int q_warp = blockIdx.x * kRxBlock + warp * kRxPerWarp;
    constexpr int R = kRxPerWarp / 32;
    int key[R], loc[R], val[R];
    unsigned peers[R];
    // loads and digit matches of all rounds first (independent), then the
    // per-warp digit counts round by round
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int q = q_warp + r * 32 + lane;
        const bool ok = q < n;
        key[r] = ok ? rx_key(keys_in, q, sentinel) : 0;
        val[r] = ok ? (vals_in ? vals_in[q] : q) : 0;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const bool ok = q_warp + r * 32 + lane < n;
        peers[r] = __match_any_sync(0xffffffffu, ok ? (key[r] >> shift) & (buckets - 1) : -1);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const bool ok = q_warp + r * 32 + lane < n;
        const int d = (key[r] >> shift) & (buckets - 1);
        const int rank = __popc(peers[r] & ((1u << lane) - 1u));
        const int pre = ok ? whist[warp][d] : 0;
        __syncwarp();
        if (ok && rank == 0) whist[warp][d] = pre + __popc(peers[r]);
        __syncwarp();
        loc[r] = pre + rank;
    }
    __syncthreads();
    for (int d = threadIdx.x; d < buckets; d += kRxThreads) {
        int acc = base_s[d];
#pragma unroll
        for (int w = 0; w < kRxWarps; ++w) {
            const int t = whist[w][d];
            whist[w][d] = acc;
            acc += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int q = q_warp + r * 32 + lane;
        if (q < n) {
            const int pos = whist[warp][(key[r] >> shift) & (buckets - 1)] + loc[r];
            if (keys_out) keys_out[pos] = key[r];
            vals_out[pos] = val[r];
        }
    }
}

// items = record indices ordered by bin, then index (bins of -1 at the end).
// rec_bin and keys_tmp are overwritten; vals_tmp, counts and total are
// scratch of n, kRxMaxBuckets * ceil(n / kRxBlock) and kRxMaxBuckets ints.
int radix_bins(int n, int n_bins, int32_t *rec_bin, int32_t *keys_tmp, int32_t *vals_tmp,
               int32_t *counts, int32_t *total, int32_t *items, cudaStream_t s) {
    int bits = 1;
    while ((1 << bits) <= n_bins) ++bits;  // keys 0 .. n_bins
    const int passes = (bits + kRxMaxBits - 1) / kRxMaxBits;
    const int dbits = (bits + passes - 1) / passes;
    const int nb = (n + kRxBlock - 1) / kRxBlock;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * dbits;
        const int pb = min(dbits, bits - shift);
        const int32_t *in_keys = p == 0 ? rec_bin : (p % 2 ? keys_tmp : rec_bin);
        int32_t *out_keys = p == passes - 1 ? nullptr : (p % 2 ? rec_bin : keys_tmp);
        const int32_t *in_vals = p == 0 ? nullptr : ((passes - p) % 2 ? vals_tmp : items);
        int32_t *out_vals = (passes - 1 - p) % 2 ? vals_tmp : items;
        if (p == 0) {
            // shared memory over L1, so that more CTAs of the scatter fit on an SM
            cudaFuncSetAttribute(radix_downsweep_kernel,
                                 cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        }
        radix_upsweep_kernel<<<nb, kRxThreads, 0, s>>>(in_keys, n, n_bins, shift, pb, nb, counts);
        radix_scan_kernel<<<1 << pb, kRxScanThreads, 0, s>>>(counts, nb, total);
        radix_downsweep_kernel<<<nb, kRxThreads, 0, s>>>(in_keys, in_vals, n, n_bins, shift, pb,
                                                         nb, counts, total, out_keys, out_vals);
    }
    return sc::launch_status("radix bins");
}

// Scan, placement and sort of counted records.
int bin_finish(int n_rec, const sc::TileGeom &g, int32_t *tile_count, int32_t *rec_bin,
               const sc::BinLayout &b, int32_t *tile_start, int32_t *items, int32_t *status,
               cudaStream_t s) {
    const int n_bins = 2 * g.n_tiles;
    bin_tile_scan_kernel<<<1, kScanThreads, 0, s>>>(tile_count, n_bins, tile_start, nullptr);
    if (b.rx_vals)
        return radix_bins(n_rec, n_bins, rec_bin, b.rec_rank, b.rx_vals, b.rx_counts, b.rx_total,
                          items, s);
    const int32_t *rec_rank = b.rec_rank;
    int32_t *big = b.big;
    int grid = (n_rec + 255) / 256;
    if (grid > 152 * 8) grid = 152 * 8;
    bin_place_kernel<<<grid, 256, 0, s>>>(rec_bin, rec_rank, n_rec, tile_start, items, status);
    int rc = sc::launch_status("sc_bin_finish");
    if (rc) return rc;
    return bin_sort(n_bins, tile_start, items, big, s);
}

}  // namespace

namespace sc {

int tile_geom(const ScSplatParams *p, TileGeom &g) {
    SC_REQUIRE(p != nullptr, "splat params are NULL");
    SC_REQUIRE(p->tile == 8 || p->tile == 16 || p->tile == 32, "tile=%d must be 8, 16 or 32",
               p->tile);
    SC_REQUIRE(p->warps == 1 || p->warps == 2 || p->warps == 4 || p->warps == 8,
               "warps=%d must be 1, 2, 4 or 8", p->warps);
    SC_REQUIRE(p->halo >= 1 && p->halo <= 512, "halo=%d out of range", p->halo);
    SC_REQUIRE(p->nw > 0 && p->nh > 0, "image size %dx%d", p->nw, p->nh);
    SC_REQUIRE(p->tiles_x == (p->nw + p->tile - 1) / p->tile &&
                   p->tiles_y == (p->nh + p->tile - 1) / p->tile,
               "tiles_x/tiles_y inconsistent with image and tile size");
    SC_REQUIRE(p->n_images >= 1, "n_images=%d", p->n_images);
    g.tile = p->tile;
    g.halo = p->halo;
    g.edge = p->tile + p->halo;
    g.warps = p->warps;
    g.tiles_x = p->tiles_x;
    g.tiles_y = p->tiles_y;
    g.tiles_per_image = p->tiles_x * p->tiles_y;
    g.n_tiles = g.tiles_per_image * p->n_images;
    g.nw = p->nw;
    g.nh = p->nh;
    g.rec_per_image = p->rec_per_image;
    g.n_images = p->n_images;
    SC_REQUIRE(g.n_tiles <= (1 << 24), "too many tiles (%d) in one launch", g.n_tiles);
    return SC_OK;
}

int bin_layout(const TileGeom &g, int n_rec, void *d_ws, size_t ws_bytes, BinLayout &b) {
    const int n_bins = 2 * g.n_tiles;
    b.count = static_cast<int32_t *>(d_ws);
    b.cursor = b.count + n_bins;
    const bool full = ws_bytes >= sc_bin_workspace_bytes(n_rec, g.n_tiles);
    b.rec_bin = full ? b.cursor + n_bins : nullptr;
    b.rec_rank = full ? b.rec_bin + n_rec : nullptr;
    b.big = full ? b.rec_rank + n_rec : nullptr;
    b.rx_vals = b.rx_counts = b.rx_total = nullptr;
    if (full && n_rec >= kRadixMinRecords) {
        uintptr_t p = reinterpret_cast<uintptr_t>(b.big + 2 * g.n_tiles + 1);
        p = (p + 15) & ~(uintptr_t)15;
        b.rx_vals = reinterpret_cast<int32_t *>(p);
        b.rx_counts = b.rx_vals + n_rec;
        b.rx_total = b.rx_counts + (size_t)kRxMaxBuckets * ((n_rec + kRxBlock - 1) / kRxBlock);
    }
    return SC_OK;
}

}  // namespace sc

// Workspace: counts and cursors of the 2 bins of every tile, then the bin and
// the rank of every record.  A workspace holding only the counts and cursors
// also works (the scatter then uses atomic cursors and recomputes each
// record's bin from its head).
static size_t bin_counts_bytes(int n_tiles_total) {
    return (size_t)4 * n_tiles_total * sizeof(int32_t);
}

extern "C" size_t sc_bin_workspace_bytes(int n_rec, int n_tiles_total) {
    if (n_rec <= 0 || n_tiles_total <= 0) return 0;
    // + the bin and rank of every record, + the list of long bins (count + bins)
    size_t bytes = bin_counts_bytes(n_tiles_total) + (size_t)2 * n_rec * sizeof(int32_t) +
                   (size_t)(2 * n_tiles_total + 1) * sizeof(int32_t);
    // + the radix sort's values, per-block digit counts and digit totals
    if (n_rec >= sc::kRadixMinRecords)
        bytes += 16 + sizeof(int32_t) * ((size_t)n_rec +
                                         (size_t)kRxMaxBuckets * ((n_rec + kRxBlock - 1) / kRxBlock) +
                                         kRxMaxBuckets);
    return bytes;
}

extern "C" int sc_bin_reset(const ScSplatParams *p, void *d_ws, size_t ws_bytes, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE_CAP(d_ws && ws_bytes >= bin_counts_bytes(g.n_tiles), "sc_bin_reset: workspace %zu < %zu",
               ws_bytes, bin_counts_bytes(g.n_tiles));
    return sc::cuda_status(cudaMemsetAsync(d_ws, 0, sizeof(int32_t) * 2 * g.n_tiles,
                                           sc::as_stream(stream)),
                           "sc_bin_reset");
}

extern "C" int sc_bin_finish(int n_rec, const ScSplatParams *p, void *d_ws, size_t ws_bytes,
                             int32_t *d_tile_start, int32_t *d_items, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(n_rec >= 0, "n_rec=%d", n_rec);
    SC_REQUIRE(d_tile_start != nullptr, "sc_bin_finish: tile_start is NULL");
    cudaStream_t s = sc::as_stream(stream);
    if (n_rec == 0)
        return sc::cuda_status(
            cudaMemsetAsync(d_tile_start, 0, sizeof(int32_t) * (2 * g.n_tiles + 1), s),
            "sc_bin_finish");
    SC_REQUIRE(d_ws && d_items, "sc_bin_finish: NULL pointer");
    SC_REQUIRE_CAP(ws_bytes >= sc_bin_workspace_bytes(n_rec, g.n_tiles),
               "sc_bin_finish: workspace %zu < %zu bytes (counts, bins and ranks)", ws_bytes,
               sc_bin_workspace_bytes(n_rec, g.n_tiles));
    sc::BinLayout b;
    sc::bin_layout(g, n_rec, d_ws, ws_bytes, b);
    return bin_finish(n_rec, g, b.count, b.rec_bin, b, d_tile_start, d_items, nullptr, s);
}

extern "C" int sc_bin_steps(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                            void *d_ws, size_t ws_bytes, int32_t *d_tile_start, int32_t *d_items,
                            int32_t *d_status, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(n_rec >= 0, "n_rec=%d", n_rec);
    SC_REQUIRE(d_tile_start != nullptr, "sc_bin_steps: tile_start is NULL");
    cudaStream_t s = sc::as_stream(stream);
    if (n_rec == 0) {
        return sc::cuda_status(
            cudaMemsetAsync(d_tile_start, 0, sizeof(int32_t) * (2 * g.n_tiles + 1), s),
            "sc_bin_steps");
    }
    SC_REQUIRE(d_recs && d_items && d_ws, "sc_bin_steps: NULL pointer");
    SC_REQUIRE_CAP(ws_bytes >= bin_counts_bytes(g.n_tiles), "sc_bin_steps: workspace %zu < %zu bytes",
               ws_bytes, bin_counts_bytes(g.n_tiles));
    SC_REQUIRE(g.rec_per_image == 0 || (int64_t)g.rec_per_image * g.n_images >= n_rec,
               "sc_bin_steps: rec_per_image too small for n_rec");
    const int n_bins = 2 * g.n_tiles;
    sc::BinLayout b;
    sc::bin_layout(g, n_rec, d_ws, ws_bytes, b);
    rc = sc::cuda_status(cudaMemsetAsync(b.count, 0, sizeof(int32_t) * n_bins, s),
                         "sc_bin_steps memset");
    if (rc) return rc;
    int grid = (n_rec + 255) / 256;
    if (grid > 152 * 8) grid = 152 * 8;
    bin_count_kernel<<<grid, 256, 0, s>>>(d_recs, n_rec, g, b.count, b.rec_bin,
                                          sc::rank_array(b), d_status);
    if (b.rec_bin)
        return bin_finish(n_rec, g, b.count, b.rec_bin, b, d_tile_start, d_items, d_status, s);
    bin_tile_scan_kernel<<<1, kScanThreads, 0, s>>>(b.count, n_bins, d_tile_start, b.cursor);
    bin_scatter_kernel<<<grid, 256, 0, s>>>(d_recs, n_rec, g, b.cursor, d_items, d_status);
    rc = sc::launch_status("sc_bin_steps");
    if (rc) return rc;
    return bin_sort(n_bins, d_tile_start, d_items, nullptr, s);
}

// ---------------------------------------------------------------------------
// sc_bin_steps_static: the same counting sort with its counts and cursors in
// a fixed device array instead of a caller workspace, for callers that have
// no device allocator to hand (a C or FFI host that is given only the record
// and output buffers) or that must not allocate per frame.
namespace {

static __device__ __align__(256) int32_t g_bin_scratch[4 * SC_BIN_STATIC_MAX_TILES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices];

// Address of g_bin_scratch on the current device, looked up once per device.
int bin_scratch(void **out) {
    int dev = -1;
    int rc = sc::cuda_status(cudaGetDevice(&dev), "sc_bin_steps_static: cudaGetDevice");
    if (rc) return rc;
    SC_REQUIRE(dev >= 0 && dev < kMaxDevices, "sc_bin_steps_static: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_ptr[dev] == nullptr) {
        void *p = nullptr;
        rc = sc::cuda_status(cudaGetSymbolAddress(&p, g_bin_scratch),
                             "sc_bin_steps_static: cudaGetSymbolAddress");
        if (rc) return rc;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SC_OK;
}

}  // namespace

extern "C" int sc_bin_steps_static(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                                   int32_t *d_tile_start, int32_t *d_items, int32_t *d_status,
                                   void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(g.n_tiles <= SC_BIN_STATIC_MAX_TILES,
               "sc_bin_steps_static: %d tiles exceed the fixed scratch of %d tiles", g.n_tiles,
               SC_BIN_STATIC_MAX_TILES);
    void *ws = nullptr;
    rc = bin_scratch(&ws);
    if (rc) return rc;
    // sc_bin_steps clears the counts on the stream before counting; the
    // cursors are written by the scan.
    return sc_bin_steps(d_recs, n_rec, p, ws, sizeof(g_bin_scratch), d_tile_start, d_items,
                        d_status, stream);
}

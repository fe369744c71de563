// i2_pairs.cu -- O(N) pair-list builder on the device, and the host helpers it shares with the
// host builder (i2_capi.cu).
//
// The reference classifies pairs on the GPU by counting shared vertex indices over all i < j
// pairs (src/Mesh3d.cu:93-142, launched from prepareMesh, src/Mesh3d.cu:243-262): O(N^2) work,
// and blocked beyond N = 46,340 cells.  Here:
//   1. vertex -> cell incidence (CSR: degree count, exclusive scan, scatter);
//   2. common-vertex / common-edge pairs: for each cell i, the cells j > i met through its three
//      vertices' incidence lists, each counted once (from the first of i's vertices that j
//      holds), classed by the number of shared vertices;
//   3. near-field disjoint pairs: centroids hashed to a uniform grid of cell edge r (sorted by
//      grid key), each cell scanning the 27 grid cells around its own; or, with no radius,
//      every disjoint j > i (one warp per row, ballot-compacted, already in order);
//   4. a count pass and a write pass per list, with exclusive scans giving each row's offset,
//      then a radix sort of the (i, j) keys so the lists come out in (i, j) order whatever the
//      order of the atomics in step 1.
// Scans and sorts are CUB's; everything else is below.
#include "i2_pairs.h"

#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace i2 {

// ------------------------------------------------------------------ shared host helpers
int edge_sum_shift(double max_len, long long half_edges)
{
    int em = 0;
    std::frexp(max_len, &em);  // max_len < 2^em
    int en = 0;
    while ((1LL << en) < half_edges) ++en;
    return 62 - em - en;
}

namespace {

inline double host_edge_length(const double *V, int a, int b)
{
    const double *p = V + 3LL * a, *q = V + 3LL * b;
    const double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

} // namespace

double mean_edge_length(const double *V, const int *C, int nc)
{
    std::vector<std::pair<int, int>> edges;
    edges.reserve(3LL * nc);
    for (int c = 0; c < nc; ++c)
        for (int d = 0; d < 3; ++d) {
            int a = C[3 * c + d], b = C[3 * c + (d + 1) % 3];
            if (a > b) std::swap(a, b);
            edges.emplace_back(a, b);
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    double mx = 0.0;
    for (auto &e : edges) mx = std::max(mx, host_edge_length(V, e.first, e.second));
    if (edges.empty() || mx == 0.0) return 0.0;
    const int shift = edge_sum_shift(mx, 3LL * nc);
    const double scale = std::ldexp(1.0, shift);
    unsigned long long sum = 0;
    for (auto &e : edges) sum += (unsigned long long)std::llrint(host_edge_length(V, e.first, e.second) * scale);
    return std::ldexp((double)sum, -shift) / (double)edges.size();
}

NearGrid near_grid(const double *centres, int nc, double r)
{
    NearGrid g;
    g.r = r;
    g.r2 = r * r;
    double hi[3] = {-1e300, -1e300, -1e300};
    for (int d = 0; d < 3; ++d) g.lo[d] = 1e300;
    for (int c = 0; c < nc; ++c)
        for (int d = 0; d < 3; ++d) {
            g.lo[d] = std::min(g.lo[d], centres[3 * c + d]);
            hi[d] = std::max(hi[d], centres[3 * c + d]);
        }
    for (int d = 0; d < 3; ++d) g.dims[d] = std::max(1LL, std::min(1LL << 20, (long long)std::floor((hi[d] - g.lo[d]) / r) + 1));
    return g;
}

// ------------------------------------------------------------------ device side
namespace {

constexpr int kTpb = 256;

int grid_for(long long n, int tpb = kTpb) { return (int)std::max(1LL, (n + tpb - 1) / tpb); }

// |V_a - V_b| with the host's operation order and no fused multiply-adds
__device__ __forceinline__ double dev_edge_length(const double *__restrict__ V, int a, int b)
{
    const double dx = V[3LL * a] - V[3LL * b], dy = V[3LL * a + 1] - V[3LL * b + 1], dz = V[3LL * a + 2] - V[3LL * b + 2];
    return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

__device__ __forceinline__ double dev_dist2(const double *__restrict__ ctr, int i, int j)
{
    const double dx = ctr[3LL * i] - ctr[3LL * j], dy = ctr[3LL * i + 1] - ctr[3LL * j + 1], dz = ctr[3LL * i + 2] - ctr[3LL * j + 2];
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ int holds(int v, int3 c) { return (v == c.x) + (v == c.y) + (v == c.z); }

__device__ __forceinline__ int3 cell(const int *__restrict__ C, int c) { return make_int3(C[3LL * c], C[3LL * c + 1], C[3LL * c + 2]); }

// half-edge keys (min vertex * nv + max vertex) and the largest edge length (non-negative
// doubles order like their bit patterns)
__global__ void k_half_edges(int nc, int nv, const int *__restrict__ C, const double *__restrict__ V, unsigned long long *keys,
                             unsigned long long *max_bits)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double len = 0.0;
    if (k < 3LL * nc) {
        const long long c = k / 3;
        const int d = (int)(k - 3 * c);
        int a = C[3 * c + d], b = C[3 * c + (d + 1) % 3];
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        keys[k] = (unsigned long long)a * (unsigned long long)nv + (unsigned long long)b;
        len = dev_edge_length(V, a, b);
    }
    unsigned long long bits = (unsigned long long)__double_as_longlong(len);
    for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, bits);
}

// fixed-point sum and count of the unique edges (sorted half-edge keys)
__global__ void k_edge_sum(long long n, int nv, const unsigned long long *__restrict__ keys, const double *__restrict__ V, double scale,
                           unsigned long long *sum, unsigned long long *count)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long term = 0, uniq = 0;
    if (k < n && (k == 0 || keys[k - 1] != keys[k])) {
        const int a = (int)(keys[k] / (unsigned long long)nv), b = (int)(keys[k] % (unsigned long long)nv);
        term = (unsigned long long)llrint(dev_edge_length(V, a, b) * scale);
        uniq = 1;
    }
    for (int off = 16; off > 0; off >>= 1) {
        term += __shfl_xor_sync(0xffffffffu, term, off);
        uniq += __shfl_xor_sync(0xffffffffu, uniq, off);
    }
    if ((threadIdx.x & 31) == 0 && uniq) {
        atomicAdd(sum, term);
        atomicAdd(count, uniq);
    }
}

__global__ void k_vertex_degree(long long n3, const int *__restrict__ C, int *deg)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n3) atomicAdd(&deg[C[k]], 1);
}

__global__ void k_vertex_fill(long long n3, const int *__restrict__ C, int *fill, int *inc)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n3) inc[atomicAdd(&fill[C[k]], 1)] = (int)(k / 3);
}

struct GridArgs {
    double lo[3];
    double r;
    long long dims[3];
};

__device__ __forceinline__ void grid_cell(const GridArgs &G, const double *__restrict__ ctr, int c, long long &x, long long &y, long long &z)
{
    x = min(G.dims[0] - 1, (long long)((ctr[3LL * c] - G.lo[0]) / G.r));
    y = min(G.dims[1] - 1, (long long)((ctr[3LL * c + 1] - G.lo[1]) / G.r));
    z = min(G.dims[2] - 1, (long long)((ctr[3LL * c + 2] - G.lo[2]) / G.r));
}

__global__ void k_grid_keys(int nc, const double *__restrict__ ctr, GridArgs G, unsigned long long *gk, int *gv)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    long long x, y, z;
    grid_cell(G, ctr, c, x, y, z);
    gk[c] = (unsigned long long)((x * G.dims[1] + y) * G.dims[2] + z);
    gv[c] = c;
}

struct BuildArgs {
    int nc;
    const int *C;
    const double *ctr;
    const int *inc_off, *inc;         // vertex -> incident cells
    const unsigned long long *gk;     // grid keys, sorted
    const int *gv;                    // cells in grid-key order
    GridArgs G;
    double r2;
    int mode;                         // 0: no disjoint list, 1: near field, 2: every disjoint pair
    long long *cnt[3];                // count pass: pairs j > i per cell (vertex, edge, disjoint)
    const long long *off[3];          // write pass: first slot of each cell's row
    unsigned long long *out[3];       // write pass: keys i * nc + j
};

__device__ __forceinline__ long long lower_bound_u64(const unsigned long long *__restrict__ a, long long n, unsigned long long key)
{
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// one thread per cell i: its common-vertex and common-edge partners j > i and, in near-field
// mode, its disjoint partners j > i within the radius
template <bool WRITE>
__global__ void __launch_bounds__(kTpb) k_cell_pairs(BuildArgs B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.nc) return;
    const int3 ci = cell(B.C, i);
    const int iv[3] = {ci.x, ci.y, ci.z};
    const unsigned long long row = (unsigned long long)i * (unsigned long long)B.nc;
    long long nvx = 0, ned = 0, nfar = 0, ntouch = 0;
    for (int d = 0; d < 3; ++d) {
        const int v = iv[d];
        for (int q = B.inc_off[v]; q < B.inc_off[v + 1]; ++q) {
            const int j = B.inc[q];
            if (j <= i) continue;
            const int3 cj = cell(B.C, j);
            bool earlier = false;
            for (int e = 0; e < d; ++e) earlier = earlier || holds(iv[e], cj) > 0;
            if (earlier) continue;  // j was met through an earlier vertex of i
            const int shared = (holds(iv[0], cj) > 0) + (holds(iv[1], cj) > 0) + (holds(iv[2], cj) > 0);
            ++ntouch;
            if (shared == 1) {
                if (WRITE) B.out[0][B.off[0][i] + nvx] = row + j;
                ++nvx;
            } else if (shared == 2) {
                if (WRITE) B.out[1][B.off[1][i] + ned] = row + j;
                ++ned;
            }
        }
    }
    if (B.mode == 1) {
        long long x0, y0, z0;
        grid_cell(B.G, B.ctr, i, x0, y0, z0);
        for (long long dx = -1; dx <= 1; ++dx)
            for (long long dy = -1; dy <= 1; ++dy)
                for (long long dz = -1; dz <= 1; ++dz) {
                    const long long x = x0 + dx, y = y0 + dy, z = z0 + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= B.G.dims[0] || y >= B.G.dims[1] || z >= B.G.dims[2]) continue;
                    const unsigned long long key = (unsigned long long)((x * B.G.dims[1] + y) * B.G.dims[2] + z);
                    for (long long p = lower_bound_u64(B.gk, B.nc, key); p < B.nc && B.gk[p] == key; ++p) {
                        const int j = B.gv[p];
                        if (j <= i || !(dev_dist2(B.ctr, i, j) < B.r2)) continue;
                        const int3 cj = cell(B.C, j);
                        if (holds(iv[0], cj) || holds(iv[1], cj) || holds(iv[2], cj)) continue;
                        if (WRITE) B.out[2][B.off[2][i] + nfar] = row + j;
                        ++nfar;
                    }
                }
    }
    if (!WRITE) {
        B.cnt[0][i] = nvx;
        B.cnt[1][i] = ned;
        B.cnt[2][i] = B.mode == 2 ? (long long)(B.nc - 1 - i) - ntouch : (B.mode == 1 ? nfar : 0);
    }
}

// every disjoint pair (i, j > i): one warp per row, the lanes over 32 consecutive j at a time,
// ballot-compacted so the row comes out in j order
__global__ void __launch_bounds__(kTpb) k_all_disjoint(int nc, const int *__restrict__ C, const long long *__restrict__ off, int2 *rows)
{
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nc; i += nwarps) {
        const int3 ci = cell(C, (int)i);
        long long pos = off[i];
        for (long long base = i + 1; base < nc; base += 32) {
            const long long j = base + lane;
            bool ok = false;
            if (j < nc) {
                const int3 cj = cell(C, (int)j);
                ok = !(holds(ci.x, cj) || holds(ci.y, cj) || holds(ci.z, cj));
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) rows[pos + __popc(m & ((1u << lane) - 1u))] = make_int2((int)i, (int)j);
            pos += __popc(m);
        }
    }
}

__global__ void k_decode(long long n, int nc, const unsigned long long *__restrict__ keys, int2 *rows)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) rows[k] = make_int2((int)(keys[k] / (unsigned long long)nc), (int)(keys[k] % (unsigned long long)nc));
}

__global__ void k_self_rows(int nc, int2 *rows)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) rows[c] = make_int2(c, c);
}

int key_bits(unsigned long long max_key)
{
    int b = 1;
    while (b < 64 && (max_key >> b) != 0) ++b;
    return b;
}

// CUB scratch of at least `bytes`; a larger buffer replaces the old one only after the work
// already enqueued (which may still read it) has finished
void scratch(DevBuf<unsigned char> &tmp, size_t bytes, cudaStream_t s)
{
    if (tmp.ptr && bytes <= tmp.count) return;
    I2_CHECK_CUDA(cudaStreamSynchronize(s));
    tmp.reserve(std::max<size_t>(bytes, 1));
}

// exclusive scan of n values
template <class T>
void exclusive_scan(DevBuf<unsigned char> &tmp, const T *in, T *out, long long n, cudaStream_t s)
{
    size_t bytes = 0;
    I2_CHECK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, s));
    scratch(tmp, bytes, s);
    I2_CHECK_CUDA(cub::DeviceScan::ExclusiveSum(tmp.ptr, bytes, in, out, n, s));
}

void sort_keys(DevBuf<unsigned char> &tmp, unsigned long long *keys, unsigned long long *alt, long long n, int end_bit,
               unsigned long long *&sorted, cudaStream_t s)
{
    cub::DoubleBuffer<unsigned long long> db(keys, alt);
    size_t bytes = 0;
    I2_CHECK_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, bytes, db, n, 0, end_bit, s));
    scratch(tmp, bytes, s);
    I2_CHECK_CUDA(cub::DeviceRadixSort::SortKeys(tmp.ptr, bytes, db, n, 0, end_bit, s));
    sorted = db.Current();
}

} // namespace

void build_pair_lists_device(const double *V, const int *C, const double *centres, int nv, int nc, const double *dV, const int *dC,
                             double near_factor, DevicePairLists &out, cudaStream_t s)
{
    const long long n3 = 3LL * nc;
    DevBuf<unsigned char> tmp;
    // 1. vertex -> cell incidence
    DevBuf<int> deg, inc_off, fill, inc;
    deg.reserve(nv + 1);
    inc_off.reserve(nv + 1);
    fill.reserve(nv + 1);
    inc.reserve(std::max<long long>(n3, 1));
    I2_CHECK_CUDA(cudaMemsetAsync(deg.ptr, 0, (nv + 1) * sizeof(int), s));
    k_vertex_degree<<<grid_for(n3), kTpb, 0, s>>>(n3, dC, deg.ptr);
    exclusive_scan(tmp, deg.ptr, inc_off.ptr, nv + 1, s);
    I2_CHECK_CUDA(cudaMemcpyAsync(fill.ptr, inc_off.ptr, (nv + 1) * sizeof(int), cudaMemcpyDeviceToDevice, s));
    k_vertex_fill<<<grid_for(n3), kTpb, 0, s>>>(n3, dC, fill.ptr, inc.ptr);

    BuildArgs B{};
    B.nc = nc;
    B.C = dC;
    B.inc_off = inc_off.ptr;
    B.inc = inc.ptr;
    B.mode = near_factor > 0 ? 1 : 2;
    DevBuf<double> dctr;
    DevBuf<unsigned long long> gk, gk_alt;
    DevBuf<int> gv, gv_alt;
    if (near_factor > 0) {
        // 2. near-field radius: fixed-point mean over the unique edges
        DevBuf<unsigned long long> he, he_alt, acc;
        he.reserve(n3);
        he_alt.reserve(n3);
        acc.reserve(3);
        I2_CHECK_CUDA(cudaMemsetAsync(acc.ptr, 0, 3 * sizeof(unsigned long long), s));
        k_half_edges<<<grid_for(n3), kTpb, 0, s>>>(nc, nv, dC, dV, he.ptr, acc.ptr);
        unsigned long long *hs = nullptr;
        sort_keys(tmp, he.ptr, he_alt.ptr, n3, key_bits((unsigned long long)nv * (unsigned long long)nv), hs, s);
        unsigned long long max_bits = 0;
        I2_CHECK_CUDA(cudaMemcpyAsync(&max_bits, acc.ptr, sizeof max_bits, cudaMemcpyDeviceToHost, s));
        I2_CHECK_CUDA(cudaStreamSynchronize(s));
        double mx;
        std::memcpy(&mx, &max_bits, sizeof mx);
        double mean = 0.0;
        if (mx > 0.0) {
            const int shift = edge_sum_shift(mx, n3);
            k_edge_sum<<<grid_for(n3), kTpb, 0, s>>>(n3, nv, hs, dV, std::ldexp(1.0, shift), acc.ptr + 1, acc.ptr + 2);
            unsigned long long sc[2];
            I2_CHECK_CUDA(cudaMemcpyAsync(sc, acc.ptr + 1, sizeof sc, cudaMemcpyDeviceToHost, s));
            I2_CHECK_CUDA(cudaStreamSynchronize(s));
            if (sc[1]) mean = std::ldexp((double)sc[0], -shift) / (double)sc[1];
        }
        const double r = near_factor * mean;
        if (r > 0.0) {
            // 3. centroid grid, sorted by grid key
            const NearGrid g = near_grid(centres, nc, r);
            for (int d = 0; d < 3; ++d) {
                B.G.lo[d] = g.lo[d];
                B.G.dims[d] = g.dims[d];
            }
            B.G.r = g.r;
            B.r2 = g.r2;
            dctr.reserve(3LL * nc);
            I2_CHECK_CUDA(cudaMemcpyAsync(dctr.ptr, centres, 3LL * nc * sizeof(double), cudaMemcpyHostToDevice, s));
            gk.reserve(nc);
            gk_alt.reserve(nc);
            gv.reserve(nc);
            gv_alt.reserve(nc);
            k_grid_keys<<<grid_for(nc), kTpb, 0, s>>>(nc, dctr.ptr, B.G, gk.ptr, gv.ptr);
            cub::DoubleBuffer<unsigned long long> dk(gk.ptr, gk_alt.ptr);
            cub::DoubleBuffer<int> dv(gv.ptr, gv_alt.ptr);
            const int bits = key_bits((unsigned long long)(g.dims[0] * g.dims[1] * g.dims[2]));
            size_t bytes = 0;
            I2_CHECK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, dk, dv, nc, 0, bits, s));
            scratch(tmp, bytes, s);
            I2_CHECK_CUDA(cub::DeviceRadixSort::SortPairs(tmp.ptr, bytes, dk, dv, nc, 0, bits, s));
            B.gk = dk.Current();
            B.gv = dv.Current();
            B.ctr = dctr.ptr;
        } else {
            B.mode = 0;
        }
    } else {
        I2_REQUIRE((long long)nc * nc <= 4000000000LL, I2_ERR_UNSUPPORTED, "all-pairs lists above 63k cells are not supported");
    }

    // 4. count pass, row offsets, write pass
    DevBuf<long long> cnt[3], off[3];
    for (int k = 0; k < 3; ++k) {
        cnt[k].reserve(nc + 1LL);
        off[k].reserve(nc + 1LL);
        I2_CHECK_CUDA(cudaMemsetAsync(cnt[k].ptr + nc, 0, sizeof(long long), s));
        B.cnt[k] = cnt[k].ptr;
    }
    k_cell_pairs<false><<<grid_for(nc), kTpb, 0, s>>>(B);
    long long total[3];
    for (int k = 0; k < 3; ++k) {
        exclusive_scan(tmp, cnt[k].ptr, off[k].ptr, nc + 1LL, s);
        I2_CHECK_CUDA(cudaMemcpyAsync(&total[k], off[k].ptr + nc, sizeof(long long), cudaMemcpyDeviceToHost, s));
        B.off[k] = off[k].ptr;
    }
    I2_CHECK_CUDA(cudaStreamSynchronize(s));
    DevBuf<unsigned long long> keys[3], alt;
    long long most = 0;
    for (int k = 0; k < 3; ++k) {
        const bool keyed = k < 2 || B.mode == 1;
        if (keyed) keys[k].reserve(std::max(total[k], 1LL));
        B.out[k] = keyed ? keys[k].ptr : nullptr;
        if (keyed) most = std::max(most, total[k]);
    }
    k_cell_pairs<true><<<grid_for(nc), kTpb, 0, s>>>(B);
    // 5. (i, j) order: radix sort of the keys, then (i, j) rows
    alt.reserve(std::max(most, 1LL));
    const int cls_of[3] = {I2_SIMPLE_NEIGHBORS, I2_ATTACHED_NEIGHBORS, I2_NOT_NEIGHBORS};
    const int bits = key_bits((unsigned long long)nc * (unsigned long long)nc);
    for (int k = 0; k < 3; ++k) {
        const int cls = cls_of[k];
        out.n[cls] = total[k];
        out.rows[cls].release();
        out.rows[cls].reserve(std::max(total[k], 1LL));
        if (total[k] == 0) continue;
        if (k == 2 && B.mode == 2) {
            k_all_disjoint<<<std::min(grid_for(32LL * nc), 152 * 64), kTpb, 0, s>>>(nc, dC, off[2].ptr, out.rows[cls].ptr);
            continue;
        }
        unsigned long long *sorted = nullptr;
        sort_keys(tmp, keys[k].ptr, alt.ptr, total[k], bits, sorted, s);
        k_decode<<<grid_for(total[k]), kTpb, 0, s>>>(total[k], nc, sorted, out.rows[cls].ptr);
    }
    out.n[I2_SELF] = nc;
    out.rows[I2_SELF].release();
    out.rows[I2_SELF].reserve(nc);
    k_self_rows<<<grid_for(nc), kTpb, 0, s>>>(nc, out.rows[I2_SELF].ptr);
    I2_CHECK_CUDA(cudaGetLastError());
    I2_CHECK_CUDA(cudaStreamSynchronize(s));
}

} // namespace i2

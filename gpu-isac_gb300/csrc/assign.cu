// assign.cu -- equal-size assignment of particles to groups on the peak matrix
// d[ref][particle] the multi-reference alignment writes: the step ISAC runs
// right after the alignment (bin/sp_isac2_gpu.py:1114-1136, through EMAN2's
// Util::assign_groups on the host, after d has been copied off the GPU).
//
// The host algorithm takes (reference, particle) pairs in descending peak
// order (equal peaks: smaller pair index ref*nima + particle first) and puts a
// particle into the pair's group while the group has room: maxasi = nima/nref
// places, except the group that closes last, which also takes the
// nima % nref particles left over.  With a strict order on the pairs, that
// greedy result is the unique stable assignment of the ranking with capacity
// maxasi per group (no particle and group outside it prefer each other to
// their partners), which deferred acceptance finds in parallel:
//   round:  every unplaced particle proposes to its best group among those
//           whose threshold its pair beats (a scan of its column of d); every
//           group that received proposals keeps its maxasi best pairs, its
//           threshold becomes the maxasi-th best pair key, and the rest are
//           unplaced again;
//   end:    when a round turns nobody away.  Every group then holds maxasi
//           particles; the one with the lowest threshold is the group the host
//           algorithm closes last, and the leftover particles join it.
// The result also comes out as the host function's list: each group's members
// in descending pair order, group after group, the leftovers in descending
// order of their pair with the last group, then that group's index.
//
// Pair keys are 64-bit: the peak's float bits mapped to an unsigned order
// (-0 taken as +0) above 0xFFFFFFFF - (ref*nima + particle), so that a larger
// key is an earlier pair; key 0 means "open" for a group threshold.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/gpu_aln_pack.h"
#include "gpuisac_kernels.h"
#include "host_geometry.h"

namespace gpuisac {
namespace {

constexpr unsigned kRows = 8;         // row slices of d per particle in the proposal scan
constexpr unsigned kSelThreads = 256; // threads of a group's selection / ranking CTA
constexpr unsigned kSmallSel = 1024;  // groups up to this many candidates select in shared memory
constexpr unsigned kSparseDiv = 8;    // a round with at most nima / 8 particles to place uses the list form
constexpr unsigned kErrNaN = 1u, kErrInternal = 2u;

enum { kScNext = 0, kScErr = 1, kScLast = 2, kScLeft = 3, kScCount = 4 };

__device__ __forceinline__ uint64_t pair_key(float v, uint32_t l)
{
    uint32_t u = __float_as_uint(v == 0.0f ? 0.0f : v);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((uint64_t)u << 32) | (uint64_t)(0xFFFFFFFFu - l);
}

// Each unplaced particle's best pair among the groups whose threshold it
// beats.  Block = 32 consecutive particles x kRows row slices; the lanes of a
// warp read one row of d for the block's unplaced particles, so that a round
// with few of them touches only the 32-byte sectors they share; a block with
// none returns at once.  redo = NULL: every particle (the first round);
// otherwise redo[p] = 1 marks the particles turned away last round (cleared
// here).
__global__ void __launch_bounds__(32 * kRows)
propose_kernel(const float* __restrict__ d, size_t pitch, unsigned nref, unsigned nima,
               unsigned char* __restrict__ redo, const uint64_t* __restrict__ theta, int* __restrict__ assign,
               uint64_t* __restrict__ pkey, unsigned* __restrict__ cnt, unsigned* __restrict__ touched,
               unsigned* __restrict__ err)
{
    __shared__ uint64_t s_key[kRows][32];
    __shared__ int s_grp[kRows][32];
    const unsigned x = threadIdx.x, y = threadIdx.y;
    const unsigned p = blockIdx.x * 32 + x;
    const bool live = p < nima && (!redo || redo[p]);
    if (!__syncthreads_or(live))
        return;
    if (live && redo && y == 0)
        redo[p] = 0;
    uint64_t best = 0;
    int bg = -1;
    bool nan = false;
    if (live) {
        const float* col = d + p;
#pragma unroll 4
        for (unsigned g = y; g < nref; g += kRows) {
            const float v = __ldg(col + (size_t)g * pitch);
            nan |= (v != v);
            const uint64_t k = pair_key(v, g * nima + p);
            if (k > best && k > __ldg(theta + g)) {
                best = k;
                bg = (int)g;
            }
        }
    }
    if (nan)
        atomicOr(err, kErrNaN);
    s_key[y][x] = best;
    s_grp[y][x] = bg;
    __syncthreads();
    if (y == 0 && live) {
#pragma unroll
        for (unsigned r = 1; r < kRows; r++)
            if (s_key[r][x] > best) {
                best = s_key[r][x];
                bg = s_grp[r][x];
            }
        assign[p] = bg;
        pkey[p] = best;
        if (bg >= 0) {
            atomicAdd(cnt + bg, 1u);
            touched[bg] = 1u;
        }
    }
}

// The list form of the proposal scan, for rounds with few particles to
// place: one warp per particle of list[0..n), its lanes striding over the
// rows of the particle's column, the best pair found by a warp reduction.
__global__ void __launch_bounds__(256)
propose_list_kernel(const float* __restrict__ d, size_t pitch, unsigned nref, unsigned nima,
                    const unsigned* __restrict__ list, unsigned n, unsigned char* __restrict__ redo,
                    const uint64_t* __restrict__ theta, int* __restrict__ assign, uint64_t* __restrict__ pkey,
                    unsigned* __restrict__ cnt, unsigned* __restrict__ touched, unsigned* __restrict__ err)
{
    const unsigned lane = threadIdx.x & 31;
    const unsigned i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n)
        return;
    const unsigned p = list[i];
    uint64_t best = 0;
    int bg = -1;
    bool nan = false;
    const float* col = d + p;
#pragma unroll 4
    for (unsigned g = lane; g < nref; g += 32) {
        const float v = __ldg(col + (size_t)g * pitch);
        nan |= (v != v);
        const uint64_t k = pair_key(v, g * nima + p);
        if (k > best && k > __ldg(theta + g)) {
            best = k;
            bg = (int)g;
        }
    }
#pragma unroll
    for (unsigned o = 16; o > 0; o >>= 1) {
        const uint64_t ok = __shfl_xor_sync(0xFFFFFFFFu, best, o);
        const int og = __shfl_xor_sync(0xFFFFFFFFu, bg, o);
        if (ok > best) {
            best = ok;
            bg = og;
        }
    }
    if (__any_sync(0xFFFFFFFFu, nan) && lane == 0)
        atomicOr(err, kErrNaN);
    if (lane == 0) {
        redo[p] = 0;
        assign[p] = bg;
        pkey[p] = best;
        if (bg >= 0) {
            atomicAdd(cnt + bg, 1u);
            touched[bg] = 1u;
        }
    }
}

// Exclusive scan of the member counts of the groups that received proposals
// (one CTA of 1024 threads); clears the fill counters and the next round's
// list length.
__global__ void __launch_bounds__(1024)
offsets_kernel(unsigned nref, const unsigned* __restrict__ cnt, const unsigned* __restrict__ touched,
               unsigned* __restrict__ off, unsigned* __restrict__ fill, unsigned* __restrict__ n_next)
{
    __shared__ unsigned s_warp[32];
    __shared__ unsigned s_carry;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_carry = 0;
        *n_next = 0;
    }
    __syncthreads();
    for (unsigned b = 0; b < nref; b += 1024) {
        const unsigned g = b + threadIdx.x;
        const unsigned v = (g < nref && touched[g]) ? cnt[g] : 0u;
        unsigned s = v;
#pragma unroll
        for (unsigned o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o)
                s += t;
        }
        if (lane == 31)
            s_warp[w] = s;
        __syncthreads();
        if (w == 0) {
            unsigned ws = s_warp[lane];
#pragma unroll
            for (unsigned o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(0xFFFFFFFFu, ws, o);
                if (lane >= o)
                    ws += t;
            }
            s_warp[lane] = ws;
        }
        __syncthreads();
        const unsigned incl = s + (w ? s_warp[w - 1] : 0u);
        if (g < nref) {
            off[g] = s_carry + incl - v;
            fill[g] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 1023)
            s_carry += incl;
        __syncthreads();
    }
}

// Members of the groups that received proposals, bucketed by group.
__global__ void __launch_bounds__(256)
scatter_kernel(unsigned nima, const int* __restrict__ assign, const uint64_t* __restrict__ pkey,
               const unsigned* __restrict__ touched, const unsigned* __restrict__ off, unsigned* __restrict__ fill,
               unsigned* __restrict__ bp, uint64_t* __restrict__ bk)
{
    const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nima)
        return;
    const int g = assign[p];
    if (g < 0 || !touched[g])
        return;
    const unsigned s = off[g] + atomicAdd(fill + g, 1u);
    bp[s] = p;
    bk[s] = pkey[p];
}

// The k-th largest of c distinct keys (1 <= k <= c), by a radix select over
// the 8-bit digits from the top, in one CTA; stops early once one key is left
// in the selected bucket.
__device__ uint64_t kth_largest(const uint64_t* __restrict__ keys, unsigned c, unsigned k)
{
    __shared__ unsigned hist[256];
    __shared__ uint64_t s_prefix, s_found;
    __shared__ unsigned s_k, s_single;
    uint64_t prefix = 0, mask = 0;
    unsigned kk = k;
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (unsigned i = threadIdx.x; i < 256; i += blockDim.x)
            hist[i] = 0;
        __syncthreads();
        for (unsigned i = threadIdx.x; i < c; i += blockDim.x) {
            const uint64_t v = keys[i];
            if ((v & mask) == prefix)
                atomicAdd(&hist[(unsigned)(v >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned acc = 0;
            int b = 255;
            for (; b > 0; b--) {
                if (acc + hist[b] >= kk)
                    break;
                acc += hist[b];
            }
            s_prefix = prefix | ((uint64_t)b << shift);
            s_k = kk - acc;
            s_single = hist[b] == 1u;
        }
        __syncthreads();
        prefix = s_prefix;
        mask |= 0xFFull << shift;
        kk = s_k;
        if (s_single) {
            for (unsigned i = threadIdx.x; i < c; i += blockDim.x) {
                const uint64_t v = keys[i];
                if ((v & mask) == prefix)
                    s_found = v;
            }
            __syncthreads();
            return s_found;
        }
        __syncthreads();
    }
    return prefix;
}

// The k-th largest of c <= kSmallSel distinct keys: the one with exactly
// k - 1 larger keys, counted against a copy in shared memory.
__device__ uint64_t kth_largest_small(const uint64_t* __restrict__ keys, unsigned c, unsigned k)
{
    __shared__ uint64_t s_keys[kSmallSel];
    __shared__ uint64_t s_found;
    for (unsigned i = threadIdx.x; i < c; i += blockDim.x)
        s_keys[i] = keys[i];
    __syncthreads();
    for (unsigned i = threadIdx.x; i < c; i += blockDim.x) {
        const uint64_t v = s_keys[i];
        unsigned larger = 0;
        for (unsigned j = 0; j < c; j++)
            larger += s_keys[j] > v;
        if (larger == k - 1)
            s_found = v;
    }
    __syncthreads();
    return s_found;
}

// One CTA per group: a group with proposals and at least maxasi members keeps
// its maxasi best, takes the maxasi-th best key as its threshold and turns
// the others away: marked in redo and appended to list (they propose again
// next round); n_next counts them.
__global__ void __launch_bounds__(kSelThreads)
select_kernel(unsigned maxasi, const unsigned* __restrict__ off, const unsigned* __restrict__ bp,
              const uint64_t* __restrict__ bk, unsigned* __restrict__ cnt, unsigned* __restrict__ touched,
              uint64_t* __restrict__ theta, int* __restrict__ assign, unsigned char* __restrict__ redo,
              unsigned* __restrict__ list, unsigned* __restrict__ n_next)
{
    const unsigned g = blockIdx.x;
    const unsigned t = touched[g], c = cnt[g];
    __syncthreads();
    if (!t)
        return;
    if (threadIdx.x == 0)
        touched[g] = 0;
    if (c < maxasi)
        return;
    const unsigned base = off[g];
    const uint64_t kth = c <= kSmallSel ? kth_largest_small(bk + base, c, maxasi) : kth_largest(bk + base, c, maxasi);
    if (c > maxasi)
        for (unsigned i = threadIdx.x; i < c; i += blockDim.x)
            if (bk[base + i] < kth) {
                const unsigned p = bp[base + i];
                assign[p] = -1;
                redo[p] = 1;
                list[atomicAdd(n_next, 1u)] = p;
            }
    if (threadIdx.x == 0) {
        theta[g] = kth;
        cnt[g] = maxasi;
    }
}

// The group that closed last (lowest threshold); checks that every group
// holds maxasi members.
__global__ void __launch_bounds__(1024)
last_group_kernel(unsigned nref, unsigned maxasi, const uint64_t* __restrict__ theta,
                  const unsigned* __restrict__ cnt, unsigned* __restrict__ sc)
{
    __shared__ uint64_t s_key[1024];
    __shared__ unsigned s_grp[1024];
    uint64_t best = ~0ull;
    unsigned bg = 0;
    for (unsigned g = threadIdx.x; g < nref; g += 1024) {
        if (cnt[g] != maxasi || theta[g] == 0)
            atomicOr(sc + kScErr, kErrInternal);
        if (theta[g] < best) {
            best = theta[g];
            bg = g;
        }
    }
    s_key[threadIdx.x] = best;
    s_grp[threadIdx.x] = bg;
    __syncthreads();
    for (unsigned h = 512; h > 0; h >>= 1) {
        if (threadIdx.x < h && s_key[threadIdx.x + h] < s_key[threadIdx.x]) {
            s_key[threadIdx.x] = s_key[threadIdx.x + h];
            s_grp[threadIdx.x] = s_grp[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        sc[kScLast] = s_grp[0];
        sc[kScLeft] = 0;
    }
}

// belongsto; a leftover particle joins the last group (its pair key with that
// group ranks it among the leftovers) and is tagged with group index nref.
__global__ void __launch_bounds__(256)
belong_kernel(const float* __restrict__ d, size_t pitch, unsigned nref, unsigned nima, int* __restrict__ assign,
              uint64_t* __restrict__ pkey, int* __restrict__ belongsto, unsigned* __restrict__ sc)
{
    const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nima)
        return;
    int g = assign[p];
    if (g < 0) {
        const unsigned last = sc[kScLast];
        pkey[p] = pair_key(d[(size_t)last * pitch + p], last * nima + p);
        assign[p] = (int)nref;
        atomicAdd(sc + kScLeft, 1u);
        g = (int)last;
    }
    if (belongsto)
        belongsto[p] = g;
}

// Members bucketed by final group: group g at g*maxasi, the leftovers at
// nref*maxasi (fill has nref+1 counters).
__global__ void __launch_bounds__(256)
scatter_final_kernel(unsigned nref, unsigned nima, unsigned maxasi, unsigned extra, const int* __restrict__ assign,
                     const uint64_t* __restrict__ pkey, unsigned* __restrict__ fill, unsigned* __restrict__ bp,
                     uint64_t* __restrict__ bk, unsigned* __restrict__ sc)
{
    const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nima)
        return;
    const unsigned g = (unsigned)assign[p];
    const unsigned cap = g < nref ? maxasi : extra;
    const unsigned j = atomicAdd(fill + g, 1u);
    if (g > nref || j >= cap) {
        atomicOr(sc + kScErr, kErrInternal);
        return;
    }
    const unsigned s = g * maxasi + j;
    bp[s] = p;
    bk[s] = pkey[p];
}

// Rank of each member within its group by counting the larger keys: CTA
// (g, chunk) places members chunk*256 .. +255 of group g (g = nref: the
// leftovers) at their rank.
__global__ void __launch_bounds__(kSelThreads)
rank_kernel(unsigned nref, unsigned maxasi, unsigned extra, const unsigned* __restrict__ bp,
            const uint64_t* __restrict__ bk, int* __restrict__ out, const unsigned* __restrict__ sc)
{
    __shared__ uint64_t tile[kSelThreads];
    const unsigned g = blockIdx.x;
    const unsigned c = g < nref ? maxasi : extra;
    const unsigned base = g * maxasi;
    const unsigned i = blockIdx.y * kSelThreads + threadIdx.x;
    if (blockIdx.y * kSelThreads >= c) {
        if (g == nref && blockIdx.y == 0 && threadIdx.x == 0)
            out[nref * maxasi + extra] = (int)sc[kScLast];
        return;
    }
    const bool live = i < c;
    const uint64_t ki = live ? bk[base + i] : 0;
    unsigned r = 0;
    for (unsigned j0 = 0; j0 < c; j0 += kSelThreads) {
        __syncthreads();
        if (j0 + threadIdx.x < c)
            tile[threadIdx.x] = bk[base + j0 + threadIdx.x];
        __syncthreads();
        const unsigned m = min(kSelThreads, c - j0);
        for (unsigned j = 0; j < m; j++)
            r += tile[j] > ki;
    }
    if (live)
        out[base + r] = (int)bp[base + i];
    if (g == nref && blockIdx.y == 0 && threadIdx.x == 0)
        out[nref * maxasi + extra] = (int)sc[kScLast];
}

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count)
    {
        if (count <= n)
            return cudaSuccess;
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        return e;
    }
};

struct AssignState {
    std::mutex mu;
    Buf<uint64_t> theta, pkey, bk;
    Buf<unsigned> cnt, touched, off, fill, bp, list, sc;
    Buf<unsigned char> redo;
    Buf<int> assign;
    Buf<float> d_host_copy;
    Buf<int> ids_host_copy;
    unsigned* h_sc = nullptr; // pinned
} g_asg;

int fail(int code, const char* msg)
{
    record_error(code, msg);
    return code;
}

#define A_CK(expr)                                                                                    \
    do {                                                                                              \
        cudaError_t e_ = (expr);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            char m_[384];                                                                             \
            snprintf(m_, sizeof(m_), "%s (%s) in the group assignment", cudaGetErrorString(e_), #expr); \
            return fail(1, m_);                                                                       \
        }                                                                                             \
    } while (0)

int check_args(const float* d, unsigned long long pitch, unsigned nref, unsigned nima)
{
    if (!d)
        return fail(2, "assign_groups: d is NULL");
    if (nref == 0 || nima < nref)
        return fail(2, "assign_groups: needs 1 <= nref <= nima");
    if ((unsigned long long)nref * nima > 0xFFFFFFFFull)
        return fail(2, "assign_groups: nref * nima must stay below 2^32");
    if (pitch < nima)
        return fail(2, "assign_groups: d_pitch smaller than nima");
    if ((nima / nref + kSelThreads - 1) / kSelThreads > 65535u)
        return fail(2, "assign_groups: groups of more than 16,776,960 particles");
    return 0;
}

int assign_locked(const float* d, size_t pitch, unsigned nref, unsigned nima, int* belongsto, int* id_list_long,
                  unsigned* rounds_out, cudaStream_t st)
{
    AssignState& w = g_asg;
    const unsigned maxasi = nima / nref, extra = nima % nref;
    A_CK(w.theta.ensure(nref));
    A_CK(w.cnt.ensure(nref));
    A_CK(w.touched.ensure(nref));
    A_CK(w.off.ensure(nref));
    A_CK(w.fill.ensure(nref + 1));
    A_CK(w.assign.ensure(nima));
    A_CK(w.pkey.ensure(nima));
    A_CK(w.bp.ensure(nima));
    A_CK(w.bk.ensure(nima));
    A_CK(w.redo.ensure(nima));
    A_CK(w.list.ensure(nima));
    A_CK(w.sc.ensure(kScCount));
    if (!w.h_sc)
        A_CK(cudaHostAlloc(&w.h_sc, kScCount * sizeof(unsigned), cudaHostAllocDefault));

    A_CK(cudaMemsetAsync(w.theta.p, 0, nref * sizeof(uint64_t), st));
    A_CK(cudaMemsetAsync(w.cnt.p, 0, nref * sizeof(unsigned), st));
    A_CK(cudaMemsetAsync(w.touched.p, 0, nref * sizeof(unsigned), st));
    A_CK(cudaMemsetAsync(w.sc.p, 0, kScCount * sizeof(unsigned), st));

    A_CK(cudaMemsetAsync(w.redo.p, 0, nima, st));

    const unsigned long long max_rounds = (unsigned long long)nref * nima + 1;
    unsigned rounds = 0, turned = nima;
    for (;;) {
        // the list written by the previous round's selection is read here,
        // before this round's selection rewrites it
        if (rounds > 0 && turned <= nima / kSparseDiv)
            propose_list_kernel<<<(turned + 7) / 8, 256, 0, st>>>(d, pitch, nref, nima, w.list.p, turned, w.redo.p,
                                                                  w.theta.p, w.assign.p, w.pkey.p, w.cnt.p,
                                                                  w.touched.p, w.sc.p + kScErr);
        else
            propose_kernel<<<(nima + 31) / 32, dim3(32, kRows), 0, st>>>(d, pitch, nref, nima,
                                                                          rounds ? w.redo.p : nullptr, w.theta.p,
                                                                          w.assign.p, w.pkey.p, w.cnt.p,
                                                                          w.touched.p, w.sc.p + kScErr);
        offsets_kernel<<<1, 1024, 0, st>>>(nref, w.cnt.p, w.touched.p, w.off.p, w.fill.p, w.sc.p + kScNext);
        scatter_kernel<<<(nima + 255) / 256, 256, 0, st>>>(nima, w.assign.p, w.pkey.p, w.touched.p, w.off.p,
                                                           w.fill.p, w.bp.p, w.bk.p);
        select_kernel<<<nref, kSelThreads, 0, st>>>(maxasi, w.off.p, w.bp.p, w.bk.p, w.cnt.p, w.touched.p,
                                                     w.theta.p, w.assign.p, w.redo.p, w.list.p, w.sc.p + kScNext);
        g_kernel_launches.fetch_add(4, std::memory_order_relaxed);
        A_CK(cudaGetLastError());
        A_CK(cudaMemcpyAsync(w.h_sc, w.sc.p, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        A_CK(cudaStreamSynchronize(st));
        rounds++;
        if (w.h_sc[kScErr] & kErrNaN)
            return fail(2, "assign_groups: d holds a NaN peak");
        turned = w.h_sc[kScNext];
        if (turned == 0)
            break;
        if (turned > nima || rounds >= max_rounds)
            return fail(1, "assign_groups: the proposal rounds did not settle (internal error)");
    }

    last_group_kernel<<<1, 1024, 0, st>>>(nref, maxasi, w.theta.p, w.cnt.p, w.sc.p);
    belong_kernel<<<(nima + 255) / 256, 256, 0, st>>>(d, pitch, nref, nima, w.assign.p, w.pkey.p, belongsto, w.sc.p);
    g_kernel_launches.fetch_add(2, std::memory_order_relaxed);
    if (id_list_long) {
        A_CK(cudaMemsetAsync(w.fill.p, 0, (nref + 1) * sizeof(unsigned), st));
        scatter_final_kernel<<<(nima + 255) / 256, 256, 0, st>>>(nref, nima, maxasi, extra, w.assign.p, w.pkey.p,
                                                                 w.fill.p, w.bp.p, w.bk.p, w.sc.p);
        const unsigned chunks = (std::max(std::max(maxasi, extra), 1u) + kSelThreads - 1) / kSelThreads;
        rank_kernel<<<dim3(nref + 1, chunks), kSelThreads, 0, st>>>(nref, maxasi, extra, w.bp.p, w.bk.p,
                                                                   id_list_long, w.sc.p);
        g_kernel_launches.fetch_add(2, std::memory_order_relaxed);
    }
    A_CK(cudaGetLastError());
    A_CK(cudaMemcpyAsync(w.h_sc, w.sc.p, kScCount * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    A_CK(cudaStreamSynchronize(st));
    if ((w.h_sc[kScErr] & kErrInternal) || w.h_sc[kScLeft] != extra)
        return fail(1, "assign_groups: inconsistent group sizes (internal error)");
    if (rounds_out)
        *rounds_out = rounds;
    return 0;
}

} // namespace

void assign_clear()
{
    std::lock_guard<std::mutex> lk(g_asg.mu);
    AssignState& w = g_asg;
    auto drop = [](auto& b) {
        if (b.p)
            cudaFree(b.p);
        b.p = nullptr;
        b.n = 0;
    };
    drop(w.theta), drop(w.pkey), drop(w.bk), drop(w.cnt), drop(w.touched), drop(w.off), drop(w.fill);
    drop(w.bp), drop(w.list), drop(w.sc), drop(w.redo), drop(w.assign), drop(w.d_host_copy);
    drop(w.ids_host_copy);
    if (w.h_sc)
        cudaFreeHost(w.h_sc);
    w.h_sc = nullptr;
}

} // namespace gpuisac

using namespace gpuisac;

extern "C" int gpuisac_assign_groups_device(const float* d, unsigned long long d_pitch, unsigned int nref,
                                            unsigned int nima, int* belongsto, int* id_list_long,
                                            unsigned int* rounds, void* stream)
{
    const gpuisac::NvtxRange nvtx_range("gpuisac:assign_groups");
    if (d_pitch == 0)
        d_pitch = nima;
    int rc = check_args(d, d_pitch, nref, nima);
    if (rc)
        return rc;
    if (!belongsto && !id_list_long)
        return fail(2, "assign_groups: neither belongsto nor id_list_long given");
    std::lock_guard<std::mutex> lk(g_asg.mu);
    return assign_locked(d, (size_t)d_pitch, nref, nima, belongsto, id_list_long, rounds, (cudaStream_t)stream);
}

extern "C" int gpuisac_assign_groups(const float* d, unsigned int nref, unsigned int nima, int* id_list_long)
{
    int rc = check_args(d, nima, nref, nima);
    if (rc)
        return rc;
    if (!id_list_long)
        return fail(2, "assign_groups: id_list_long is NULL");
    std::lock_guard<std::mutex> lk(g_asg.mu);
    AssignState& w = g_asg;
    const size_t n = (size_t)nref * nima;
    A_CK(w.d_host_copy.ensure(n));
    A_CK(w.ids_host_copy.ensure((size_t)nima + 1));
    A_CK(cudaMemcpy(w.d_host_copy.p, d, n * sizeof(float), cudaMemcpyHostToDevice));
    rc = assign_locked(w.d_host_copy.p, nima, nref, nima, nullptr, w.ids_host_copy.p, nullptr, nullptr);
    if (rc)
        return rc;
    A_CK(cudaMemcpy(id_list_long, w.ids_host_copy.p, ((size_t)nima + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    return 0;
}

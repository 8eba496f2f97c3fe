// Foam cluster dynamics: FoamSimulator::step (foam_dynamics.rs:172-211) with compute_forces
// (:62-94), update_connections (foam.rs:322-364) and handle_coalescence / merge_bubbles
// (foam_dynamics.rs:214-238, foam.rs:369-405) on the GPU.
//
// The reference sums the pair forces over all pairs i < j in index order (force_buffer[i] +=
// f_ij, force_buffer[j] += -f_ij), so bubble k receives, in this order: -f_jk for j < k
// ascending, its buoyancy, f_kj for j > k ascending, its drag. A pair farther apart than
// 3 (r_a + r_b) contributes exact zeros (no van der Waals, repulsion or adhesion term applies),
// and adding a zero leaves a sum unchanged. So a walk over a neighbour list sorted by bubble
// index, holding every pair that can come within that range, forms the reference's f32 sums
// exactly, in O(n) instead of O(n^2): one thread per bubble, or for small foams a few lanes that
// evaluate consecutive entries together and add them in order.
//
// Neighbour list (Verlet list): bubble k lists every j with |p_j - p_k| < 3 (r_k + r_j) + skin at
// the time of the build; it stays complete while no bubble has moved skin / 2 since (two bubbles
// close by at most twice that). The force pass checks every bubble's displacement after each step
// and flags a rebuild for the next one; merges flag one too. A rebuild bins the bubbles into a
// spatial hash of cells (edge half of 6 r_max + skin, so the 5 x 5 x 5 cells around a bubble hold
// all its candidates), counts each bubble's candidates (a warp per bubble), orders the bubbles by
// descending count, collects the candidates again into each bubble's column and sorts each column
// by index with a warp-wide bitonic sort in registers. The lists of 32 bubbles at consecutive
// positions of that order are interleaved (entry t of the bubble at position q at
// goff[q / 32] + 32 t + q % 32): the force pass reads them coalesced and, the lengths of
// neighbouring positions being nearly equal, its lanes idle little.
//
// State: per bubble float4 (x, y, z, radius) and float4 (vx, vy, vz, thickness_nm) and the id,
// double-buffered; the bubble count lives on the device (a merge changes it) and every kernel
// reads it there, so a run of steps is enqueued without host synchronisation.
//
// Arithmetic: the same f32 operations in the same order as the reference, without contraction
// (-fmad=false). glam's Vec3 (0.29.3) is component-wise f32; length() = sqrt(x*x + y*y + z*z)
// left to right; division divides each component. x^1.5 (the Hertz term) is the library's own
// evaluation from a correctly rounded square root and the exact FMA residuals of the product and
// the root (correctly rounded but for near-ties); the merged radius x^(1/3) is rounded once from
// double.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kMaxSpeed = 0.1f;   // foam_dynamics.rs:194
constexpr int kMaxCand = 2048;      // neighbour-list entries per bubble (the shared-memory sort buffer)
constexpr int kThreads = 256;
constexpr uint32_t kNone = 0xffffffffu;
constexpr unsigned long long kNoPair = ~0ull;

// kFaultWalk: a bubble's candidate walk collected a different number of entries than its count
// pass (the two passes make the same decisions, so this means a fault of the build itself).
enum Fault : uint32_t { kFaultNone = 0, kFaultCapacity = 1, kFaultDense = 2, kFaultWalk = 3 };

// Device-side control block.
struct Ctl {
    uint32_t n[2];          // bubble count; a merge pass reads n[p] and writes n[p ^ 1]
    uint32_t next_id;       // BubbleCluster::next_id
    uint32_t need_rebuild;  // set by the connection pass (displacement) and by a merge
    uint32_t go;            // the rebuild enqueued for this step runs
    uint32_t fault;         // Fault
    uint32_t steps_done;    // steps whose force pass ran in the current call
    uint32_t nconn;         // connection count after the last step (before its merge)
    unsigned long long coal_key;  // first connection (i << 32 | j) whose Weber number is over the threshold
    uint32_t merged_a, merged_b;  // ids merged by the last step, kNone if none
    float inv_cell, skin, cell, rmax;
    uint32_t list_total, dense_bubble, dense_count, pad1;
};

struct Phys {
    float surface_tension, viscosity, density, gx, gy, gz, vdw, stiffness, damping, coal_threshold;
    int coalescence;
};

struct Bufs {
    float4 *pr[2], *vt[2];  // (x, y, z, radius), (vx, vy, vz, thickness_nm)
    uint32_t *id[2];
};

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

// x^1.5 for x > 0: p = x s with s the correctly rounded sqrt(x), plus the exact FMA residuals of the
// product (x s - p) and of the root (x - s^2, scaled by x / (2 sqrt x) ~ s / 2).
__host__ __device__ __forceinline__ float pow15(float x) {
    const float s = sqrtf(x);
    const float p = x * s;
    const float e = fmaf(x, s, -p);
    const float r = fmaf(-s, s, x);
    const float c = fmaf(0.5f * r, s, e);
    return p + c;
}

// compute_interaction_force (foam_dynamics.rs:118-160) for a = the lower index: the force on a.
// far = the pair is beyond every term's range (the force is exactly zero).
__device__ __forceinline__ void pair_force(const Phys &P, float4 a, float4 b, float &fx, float &fy, float &fz) {
    fx = fy = fz = 0.0f;
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float sum_radii = a.w + b.w;
    const float three = sum_radii * 3.0f;
    // far pairs leave before the square root: with d2 above three^2 (1 + 2^-20) the rounded root
    // is at least `three`, the range where no term applies
    if (d2 > three * three * 1.00000095f) return;
    const float distance = sqrtf(d2);
    if (distance < 1e-6f) return;
    if (!(distance < three)) return;  // exact zero: no term applies (adhesion ends at 1.2 sum)
    const float ux = dx / distance, uy = dy / distance, uz = dz / distance;
    if (distance > sum_radii) {
        const float vdw = P.vdw * a.w * b.w / (distance * distance);
        fx = fx + ux * vdw;
        fy = fy + uy * vdw;
        fz = fz + uz * vdw;
    }
    const float overlap = sum_radii - distance;
    if (overlap > 0.0f) {
        const float rep = P.stiffness * pow15(overlap);
        fx = fx - ux * rep;
        fy = fy - uy * rep;
        fz = fz - uz * rep;
    }
    const float ct = sum_radii * 1.2f;
    const float md = sum_radii * 0.95f;
    if (distance < ct && distance > md) {
        const float adh = 2.0f * (ct - distance);
        fx = fx + ux * adh;
        fy = fy + uy * adh;
        fz = fz + uz * adh;
    }
}

constexpr float kCellLim = 1048574.0f;  // cell coordinates are clamped to +-(2^20 - 2)

__device__ __forceinline__ int3 cell_of(float4 p, float inv_cell) {
    return make_int3((int)floorf(fminf(fmaxf(p.x * inv_cell, -kCellLim), kCellLim)),
                     (int)floorf(fminf(fmaxf(p.y * inv_cell, -kCellLim), kCellLim)),
                     (int)floorf(fminf(fmaxf(p.z * inv_cell, -kCellLim), kCellLim)));
}

__device__ __forceinline__ uint32_t cell_hash(int x, int y, int z, uint32_t mask) {
    return ((uint32_t)x * 73856093u ^ (uint32_t)y * 19349663u ^ (uint32_t)z * 83492791u) & mask;
}

// 21 bits a coordinate: distinct for every cell of the clamped range and its neighbours.
__device__ __forceinline__ unsigned long long cell_key(int x, int y, int z) {
    return ((unsigned long long)(uint32_t)(x + (1 << 20)) << 42) |
           ((unsigned long long)(uint32_t)(y + (1 << 20)) << 21) | (unsigned long long)(uint32_t)(z + (1 << 20));
}

// A pair is listed when |p_j - p_k| < 3 (r_k + r_j) + skin.
__device__ __forceinline__ bool candidate(float4 a, float4 b, float skin) {
    const float d = len3(b.x - a.x, b.y - a.y, b.z - a.z);
    return d < (a.w + b.w) * 3.0f + skin;
}

// ----------------------------------------------------------------------------- neighbour list
struct ListArgs {
    Ctl *ctl;
    int npar;
    const float4 *pr;
    float4 *p0;             // positions at the build
    int4 *cellc;            // cell of each bubble (w: its slot in bucket order)
    uint32_t *bcount, *bstart, *bkey, *brank;
    uint32_t *bitems;       // bubbles in bucket order
    float4 *spr;            // their positions and radii, in bucket order
    unsigned long long *skey;  // their cell keys, in bucket order
    uint32_t mask;          // hash buckets - 1
    uint32_t *cnt;          // list length per bubble
    uint32_t *split;        // entries j < k of each list (the sorted list's lower part)
    uint32_t *perm;         // bubbles by descending list length: the order of the 32-bubble groups
    uint32_t *inv;          // position of each bubble in perm
    uint32_t *mhist, *mstart;  // bubbles per list length (kMaxCand + 1 bins, longest first)
    uint32_t *gcap;         // largest list length of each 32-bubble group
    uint32_t *goff;         // group offsets (ngroups + 1)
    uint32_t *nbr;          // interleaved lists
    size_t nbr_cap;
};

// Decides whether this step rebuilds (forced, or flagged by the last connection / merge pass) and
// sets the cell size from the largest radius. One block.
__global__ void __launch_bounds__(1024) list_begin_kernel(ListArgs a, int forced, float skin) {
    __shared__ float s_max[32];
    __shared__ int s_go;
    Ctl *c = a.ctl;
    if (threadIdx.x == 0) s_go = (c->fault == kFaultNone) && (forced || c->need_rebuild);
    __syncthreads();
    if (!s_go) {
        if (threadIdx.x == 0) c->go = 0;
        return;
    }
    const uint32_t n = c->n[a.npar];
    float m = 0.0f;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, a.pr[i].w);
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0.0f;
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) {
            // cells of half the largest candidate range 6 r_max + skin: the 5 x 5 x 5 cells around a
            // bubble's own hold all its candidates
            const float cell = (6.0f * m + skin) * 0.5001f + 1e-12f;
            c->inv_cell = 1.0f / cell;
            c->cell = cell;
            c->rmax = m;
            c->skin = skin;
            c->need_rebuild = 0;
            c->go = 1;
        }
    }
}

__global__ void list_bin_kernel(ListArgs a) {
    const Ctl *c = a.ctl;
    if (!c->go) return;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c->n[a.npar]) return;
    const float4 p = a.pr[k];
    const int3 q = cell_of(p, c->inv_cell);
    const uint32_t h = cell_hash(q.x, q.y, q.z, a.mask);
    a.p0[k] = p;
    a.bkey[k] = h;
    a.brank[k] = atomicAdd(a.bcount + h, 1u);
    a.cellc[k] = make_int4(q.x, q.y, q.z, 0);
}

// Exclusive scan of `count` values with one block, tile by tile (4 values a thread).
// mode 0: hash buckets (count given); mode 1: the entries of each 32-bubble group, 32 columns of its
// largest count rounded up to a multiple of 32 (count = ceil(n / 32)), with the capacity check of
// the list. (Whole 32-entry blocks per column: a group then owns exactly its share of the
// connection-bit words, word (t / 32) * 32 + lane of the group's block.)
__global__ void __launch_bounds__(1024) scan_kernel(const uint32_t *in, uint32_t *out, uint32_t count, int mode,
                                                    ListArgs a) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    Ctl *c = a.ctl;
    if (!c->go) return;
    if (mode == 1) count = (c->n[a.npar] + 31) / 32;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const uint32_t tile = blockDim.x * 4;
    for (uint32_t base = 0; base < count; base += tile) {
        uint32_t v[4], sum = 0;
        const uint32_t i0 = base + threadIdx.x * 4;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = i0 + q;
            v[q] = i < count ? (mode == 1 ? ((in[i] + 31u) & ~31u) * 32u : in[i]) : 0u;
            sum += v[q];
        }
        uint32_t x = sum;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= (unsigned)o) x += y;
        }
        if ((threadIdx.x & 31) == 31) s_w[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            uint32_t w = threadIdx.x < (blockDim.x >> 5) ? s_w[threadIdx.x] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= (unsigned)o) w += y;
            }
            s_w[threadIdx.x] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t warp_ex = (threadIdx.x >> 5) ? s_w[(threadIdx.x >> 5) - 1] : 0u;
        uint32_t run = s_carry + warp_ex + x - sum;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = i0 + q;
            if (i < count) out[i] = run;
            run += v[q];
        }
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_w[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[count] = s_carry;
        if (mode == 1) {
            c->list_total = s_carry;
            if (s_carry > a.nbr_cap) c->fault = kFaultCapacity;
        }
    }
}

// Bucket order: the bubbles of each bucket contiguous, with copies of their positions and cell
// keys, so the candidate walks read contiguous memory.
__global__ void list_scatter_kernel(ListArgs a) {
    const Ctl *c = a.ctl;
    if (!c->go) return;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c->n[a.npar]) return;
    const uint32_t slot = a.bstart[a.bkey[k]] + a.brank[k];
    const int4 q = a.cellc[k];
    a.bitems[slot] = k;
    a.spr[slot] = a.pr[k];
    a.skey[slot] = cell_key(q.x, q.y, q.z);
    a.cellc[k].w = (int)slot;
}

// Per-warp table of the cells a walk visits: slot range, cell key and the running member count.
struct CellTable {
    uint32_t s[128], n[128], pre[129];
    unsigned long long key[128];
};

// The candidate walk of one warp for bubble k. First the 5 x 5 x 5 cells around its own whose box
// comes within its largest candidate range 3 (r_k + r_max) + skin (with a margin of 1 % of a cell
// for the rounding of the cell coordinates) and whose bucket is not empty go into the table, 32
// cells at a time; then the members of all of them are swept as one range, 32 slots a round, so
// the loads of many cells are in flight together. visit(i, ok) gets every slot with ok = the slot
// holds a candidate of k (a bubble of that very cell, not k, within 3 (r_k + r_j) + skin).
template <class Visit>
__device__ __forceinline__ void walk(const ListArgs &a, const Ctl *c, float4 p, int4 q, int lane, CellTable &T,
                                     Visit &&visit) {
    const float skin = c->skin, cs = c->cell;
    const float reach = (p.w + c->rmax) * 3.0f + skin + 0.01f * cs;
    const float reach2 = reach * reach;
    uint32_t nt = 0;
    for (int c0 = 0; c0 < 125; c0 += 32) {
        const int ci = c0 + lane;
        bool use = false;
        uint32_t s0 = 0, cnt = 0;
        unsigned long long key = 0;
        if (ci < 125) {
            const int x = q.x + ci % 5 - 2, y = q.y + (ci / 5) % 5 - 2, z = q.z + ci / 25 - 2;
            const float gx = fmaxf(fmaxf(x * cs - p.x, p.x - (x + 1) * cs), 0.0f);
            const float gy = fmaxf(fmaxf(y * cs - p.y, p.y - (y + 1) * cs), 0.0f);
            const float gz = fmaxf(fmaxf(z * cs - p.z, p.z - (z + 1) * cs), 0.0f);
            if (gx * gx + gy * gy + gz * gz <= reach2) {
                const uint32_t h = cell_hash(x, y, z, a.mask);
                cnt = a.bcount[h];
                if (cnt) {
                    s0 = a.bstart[h];
                    key = cell_key(x, y, z);
                    use = true;
                }
            }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, use);
        if (use) {
            const uint32_t r = nt + __popc(bal & ((1u << lane) - 1u));
            T.s[r] = s0;
            T.n[r] = cnt;
            T.key[r] = key;
        }
        nt += __popc(bal);
    }
    __syncwarp();
    uint32_t v[4], sum = 0;  // exclusive running count over the table, 4 entries a lane
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t idx = lane * 4 + k;
        v[k] = idx < nt ? T.n[idx] : 0u;
        sum += v[k];
    }
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
    uint32_t run = x - sum;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t idx = lane * 4 + k;
        if (idx < nt) T.pre[idx] = run;
        run += v[k];
    }
    if (lane == 0) T.pre[nt] = total;
    __syncwarp();
    uint32_t cc = 0;
    for (uint32_t v0 = 0; v0 < total; v0 += 32) {
        const uint32_t vv = v0 + lane;
        bool ok = false;
        uint32_t i = 0;
        if (vv < total) {
            while (T.pre[cc + 1] <= vv) ++cc;
            i = T.s[cc] + (vv - T.pre[cc]);
            ok = i != (uint32_t)q.w && a.skey[i] == T.key[cc] && candidate(p, a.spr[i], skin);
        }
        visit(i, ok);
    }
    __syncwarp();  // the table is rebuilt for the warp's next bubble
}

// Bitonic sort of 32 R values held R per lane (element r * 32 + lane in v[r]), ascending: strides of
// 32 and more compare within a lane's registers, smaller ones across lanes by shuffles.
template <int R>
__device__ __forceinline__ void warp_sort(uint32_t (&v)[R], int lane) {
#pragma unroll
    for (int size = 2; size <= 32 * R; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                const int rs = stride >> 5;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int o = r ^ rs;
                    if (o > r) {
                        const bool up = ((r * 32) & size) == 0;
                        const uint32_t x = v[r], y = v[o];
                        v[r] = up ? min(x, y) : max(x, y);
                        v[o] = up ? max(x, y) : min(x, y);
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t y = __shfl_xor_sync(0xffffffffu, v[r], stride);
                    const bool up = (((r * 32) + lane) & size) == 0;
                    const bool low = (lane & stride) == 0;
                    v[r] = (low == up) ? min(v[r], y) : max(v[r], y);
                }
            }
        }
    }
}

constexpr int kListWarps = 4;

// Counts each bubble's candidates (a warp per bubble), and the bubbles of each count.
__global__ void __launch_bounds__(kListWarps * 32) list_count_kernel(ListArgs a) {
    __shared__ CellTable s_tab[kListWarps];
    Ctl *c = a.ctl;
    if (!c->go) return;
    const uint32_t n = c->n[a.npar];
    const int lane = threadIdx.x & 31;
    for (uint32_t k = blockIdx.x * kListWarps + (threadIdx.x >> 5); k < n; k += gridDim.x * kListWarps) {
        const float4 p = a.pr[k];
        const int4 q = a.cellc[k];
        uint32_t m = 0;
        walk(a, c, p, q, lane, s_tab[threadIdx.x >> 5],
             [&](uint32_t, bool ok) { m += __popc(__ballot_sync(0xffffffffu, ok)); });
        if (lane == 0) {
            a.cnt[k] = m;
            atomicAdd(a.mhist + (kMaxCand - min(m, (uint32_t)kMaxCand)), 1u);
            if (m > (uint32_t)kMaxCand && atomicCAS(&c->fault, kFaultNone, kFaultDense) == kFaultNone) {
                c->dense_bubble = k;
                c->dense_count = m;
            }
        }
    }
}

// Lists longer than 1024 (rare): bitonic sort in shared memory.
__device__ __noinline__ uint32_t sort_smem(uint32_t *buf, uint32_t m, uint32_t k, uint32_t *col, int lane) {
    uint32_t P = 1;
    while (P < m) P <<= 1;
    for (uint32_t t = m + lane; t < P; t += 32) buf[t] = kNone;
    __syncwarp();
    for (uint32_t size = 2; size <= P; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                const uint32_t l = i ^ stride;
                if (l > i) {
                    const uint32_t x = buf[i], y = buf[l];
                    if ((x > y) == ((i & size) == 0)) {
                        buf[i] = y;
                        buf[l] = x;
                    }
                }
            }
            __syncwarp();
        }
    uint32_t below = 0;
    for (uint32_t t = lane; t < m; t += 32) {
        col[(size_t)t * 32] = buf[t];
        below += buf[t] < k;
    }
    return below;
}

// Orders the bubbles by descending list length (counting sort over the lengths): the 32 bubbles of a
// group, which one warp of the force pass runs, then have lists of nearly the same length, and the
// longest groups start first.
__global__ void list_order_kernel(ListArgs a) {
    const Ctl *c = a.ctl;
    if (!c->go || c->fault != kFaultNone) return;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c->n[a.npar]) return;
    const uint32_t pos = atomicAdd(a.mstart + (kMaxCand - a.cnt[k]), 1u);
    a.perm[pos] = k;
    a.inv[k] = pos;
}

// The largest list length of each group of 32 consecutive positions of the order.
__global__ void list_gcap_kernel(ListArgs a) {
    const Ctl *c = a.ctl;
    if (!c->go || c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t m = t < n ? a.cnt[a.perm[t]] : 0u;
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && t < ((n + 31) & ~31u)) a.gcap[t >> 5] = m;
}

// A warp per bubble: collects the candidates again, in the walk's order, straight into the bubble's
// column (few registers: many warps hide the walk's load latency).
__global__ void __launch_bounds__(kListWarps * 32) list_walk_kernel(ListArgs a) {
    __shared__ CellTable s_tab[kListWarps];
    const Ctl *c = a.ctl;
    if (!c->go || c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const int lane = threadIdx.x & 31;
    for (uint32_t k = blockIdx.x * kListWarps + (threadIdx.x >> 5); k < n; k += gridDim.x * kListWarps) {
        const float4 p = a.pr[k];
        const int4 q = a.cellc[k];
        const uint32_t mk = a.cnt[k];  // the count pass's length: the same decisions, the same count
        const uint32_t pos = a.inv[k];
        uint32_t *col = a.nbr + a.goff[pos >> 5] + (pos & 31);
        uint32_t m = 0;
        walk(a, c, p, q, lane, s_tab[threadIdx.x >> 5], [&](uint32_t i, bool ok) {
            const uint32_t bal = __ballot_sync(0xffffffffu, ok);
            const uint32_t slot = m + __popc(bal & ((1u << lane) - 1u));
            if (ok && slot < mk) col[(size_t)slot * 32] = a.bitems[i];
            m += __popc(bal);
        });
        // a column the walk did not fill exactly would be sorted with stale entries: stop the
        // list build and every later pass of the call instead
        if (m != mk && lane == 0)
            atomicCAS(const_cast<uint32_t *>(&c->fault), (uint32_t)kFaultNone, (uint32_t)kFaultWalk);
    }
}

// Sorts the column's m entries in registers (element r * 32 + lane in v[r]) and writes them back;
// returns the number of entries below k.
template <int R>
__device__ __forceinline__ uint32_t sort_column(uint32_t *col, uint32_t m, uint32_t k, int lane) {
    uint32_t v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = r * 32 + lane;
        v[r] = e < m ? col[(size_t)e * 32] : kNone;
    }
    warp_sort<R>(v, lane);
    uint32_t below = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = r * 32 + lane;
        if (e < m) {
            col[(size_t)e * 32] = v[r];
            below += v[r] < k;
        }
    }
    return below;
}

// A warp per bubble: sorts its column by index in registers (bitonic; in shared memory beyond 1024
// entries) and records the length of its lower part.
__global__ void __launch_bounds__(kListWarps * 32, 4) list_sort_kernel(ListArgs a) {
    __shared__ uint32_t s_buf[kListWarps][kMaxCand];
    const Ctl *c = a.ctl;
    if (!c->go || c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const int lane = threadIdx.x & 31;
    uint32_t *buf = s_buf[threadIdx.x >> 5];
    for (uint32_t k = blockIdx.x * kListWarps + (threadIdx.x >> 5); k < n; k += gridDim.x * kListWarps) {
        const uint32_t m = a.cnt[k];
        const uint32_t pos = a.inv[k];
        uint32_t *col = a.nbr + a.goff[pos >> 5] + (pos & 31);
        uint32_t below;
        if (m <= 32) below = sort_column<1>(col, m, k, lane);
        else if (m <= 64) below = sort_column<2>(col, m, k, lane);
        else if (m <= 128) below = sort_column<4>(col, m, k, lane);
        else if (m <= 256) below = sort_column<8>(col, m, k, lane);
        else if (m <= 512) below = sort_column<16>(col, m, k, lane);
        else if (m <= 1024) below = sort_column<32>(col, m, k, lane);
        else {
            for (uint32_t t = lane; t < m; t += 32) buf[t] = col[(size_t)t * 32];
            __syncwarp();
            below = sort_smem(buf, m, k, col, lane);
        }
        for (int o = 16; o; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
        if (lane == 0) a.split[k] = below;
        __syncwarp();
    }
}

// ----------------------------------------------------------------------------- the step
struct DynArgs {
    Ctl *ctl;
    int npar;
    Phys P;
    float dt;
    const float4 *pr_in, *vt_in;
    const uint32_t *id_in;
    float4 *pr_out, *vt_out;
    uint32_t *id_out;
    float *force_out;  // forces-only mode: [n][3]
    const uint32_t *cnt, *split, *goff, *nbr;
    const uint32_t *perm;  // thread t of the force and connection passes runs bubble perm[t]
    uint32_t *cflag;   // connection bits, one per list entry
    const float4 *p0;
    float flag_sq;     // squared displacement from p0 beyond which the next step rebuilds (< 0: always)
};

// compute_forces + the integration of step (foam_dynamics.rs:62-94, 172-202); with force_out set,
// only the forces of the current state.
//
// L lanes per bubble (L = 1 for large foams, where one thread per bubble already fills the GPU;
// 4 or 16 for small ones, which would otherwise leave most SMs idle): the lanes evaluate the pair
// forces of L consecutive list entries at once, then every lane of the group adds the L results
// into the sum one by one in list order (shuffles), the buoyancy before the first j > k: the
// reference's sums, the same on every lane; the group's first lane writes.
template <int L>
__global__ void __launch_bounds__(kThreads, 5) forces_kernel(DynArgs a) {
    Ctl *c = a.ctl;
    if (c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t t0 = gtid / L;
    const int sub = (int)(gtid % L);
    const int lane0 = (int)(threadIdx.x & 31) - sub;
    const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << lane0);
    if (gtid == 0 && !a.force_out) {
        c->steps_done += 1;
        c->nconn = 0;
        c->coal_key = kNoPair;
        c->merged_a = c->merged_b = kNone;
    }
    if (t0 >= n) return;  // the whole group: t0 is the group's
    const uint32_t k = a.perm[t0];
    const Phys &P = a.P;
    const float4 me = a.pr_in[k];
    const float4 mv = a.vt_in[k];
    // compute_buoyancy (foam_dynamics.rs:99-113)
    const float glen = len3(P.gx, P.gy, P.gz);
    float bx, by, bz;
    {
        const float shell_volume = 4.0f * kPi * (me.w * me.w) * (mv.w * 1e-9f);
        const float film_mass = shell_volume * P.density;
        const float volume = (4.0f / 3.0f) * kPi * (me.w * (me.w * me.w));
        const float buoy = volume * 1.2f * glen;
        const float net = fmaxf(film_mass * glen - buoy, 0.0f);
        const float rcp = 1.0f / glen;
        float nx = 0.0f, ny = 0.0f, nz = 0.0f;
        if (isfinite(rcp) && rcp > 0.0f) {
            nx = P.gx * rcp;
            ny = P.gy * rcp;
            nz = P.gz * rcp;
        }
        bx = nx * net;
        by = ny * net;
        bz = nz * net;
    }
    // entries t < split are j < k, whose pair force is evaluated with j first and enters negated;
    // the buoyancy enters before the first j > k
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    const uint32_t m = a.cnt[k], split = a.split[k];
    const uint32_t *col = a.nbr + a.goff[t0 >> 5] + (t0 & 31);
    if constexpr (L == 1) {
        // one loop over the sorted list; the next entry's position fetched one iteration ahead
        float4 next = m ? a.pr_in[__ldg(col)] : me;
        for (uint32_t t = 0; t < m; ++t) {
            const float4 o = next;
            if (t + 1 < m) next = a.pr_in[__ldg(col + (size_t)(t + 1) * 32)];
            if (t == split) {
                fx = fx + bx;
                fy = fy + by;
                fz = fz + bz;
            }
            const bool lower = t < split;
            float gx, gy, gz;
            pair_force(P, lower ? o : me, lower ? me : o, gx, gy, gz);
            fx = fx + (lower ? -gx : gx);
            fy = fy + (lower ? -gy : gy);
            fz = fz + (lower ? -gz : gz);
        }
    } else {
        for (uint32_t base = 0; base < m; base += L) {
            const uint32_t t = base + sub;
            float gx = 0.0f, gy = 0.0f, gz = 0.0f;
            if (t < m) {
                const float4 o = a.pr_in[__ldg(col + (size_t)t * 32)];
                const bool lower = t < split;
                pair_force(P, lower ? o : me, lower ? me : o, gx, gy, gz);
            }
            const uint32_t cnt = min((uint32_t)L, m - base);  // the same on every lane of the group
#pragma unroll
            for (int jj = 0; jj < L; ++jj) {
                const float hx = __shfl_sync(gmask, gx, lane0 + jj);
                const float hy = __shfl_sync(gmask, gy, lane0 + jj);
                const float hz = __shfl_sync(gmask, gz, lane0 + jj);
                if ((uint32_t)jj < cnt) {
                    const uint32_t tt = base + jj;
                    if (tt == split) {
                        fx = fx + bx;
                        fy = fy + by;
                        fz = fz + bz;
                    }
                    const bool lower = tt < split;
                    fx = fx + (lower ? -hx : hx);
                    fy = fy + (lower ? -hy : hy);
                    fz = fz + (lower ? -hz : hz);
                }
            }
        }
    }
    if (split == m) {
        fx = fx + bx;
        fy = fy + by;
        fz = fz + bz;
    }
    // compute_drag (foam_dynamics.rs:163-167)
    const float drag_coeff = 6.0f * kPi * P.viscosity * me.w;
    fx = fx + (-mv.x) * drag_coeff;
    fy = fy + (-mv.y) * drag_coeff;
    fz = fz + (-mv.z) * drag_coeff;
    if (sub != 0) return;
    if (a.force_out) {
        a.force_out[3 * (size_t)k] = fx;
        a.force_out[3 * (size_t)k + 1] = fy;
        a.force_out[3 * (size_t)k + 2] = fz;
        return;
    }
    // semi-implicit Euler (foam_dynamics.rs:181-202)
    const float shell_volume = 4.0f * kPi * (me.w * me.w) * (mv.w * 1e-9f);
    const float mass = fmaxf(shell_volume * P.density, 1e-9f);
    float vx = mv.x + (fx / mass) * a.dt, vy = mv.y + (fy / mass) * a.dt, vz = mv.z + (fz / mass) * a.dt;
    vx = vx * P.damping;
    vy = vy * P.damping;
    vz = vz * P.damping;
    const float speed = len3(vx, vy, vz);
    if (speed > kMaxSpeed) {
        const float s = kMaxSpeed / speed;
        vx = vx * s;
        vy = vy * s;
        vz = vz * s;
    }
    const float4 np_ = make_float4(me.x + vx * a.dt, me.y + vy * a.dt, me.z + vz * a.dt, me.w);
    a.pr_out[k] = np_;
    a.vt_out[k] = make_float4(vx, vy, vz, mv.w);
    a.id_out[k] = a.id_in[k];
    // the neighbour list's displacement check on the new position (see connections_kernel)
    const float4 q0 = a.p0[k];
    const float ddx = np_.x - q0.x, ddy = np_.y - q0.y, ddz = np_.z - q0.z;
    if (ddx * ddx + ddy * ddy + ddz * ddz > a.flag_sq) atomicOr(&c->need_rebuild, 1u);
}

// update_connections (foam.rs:322-364) on the new positions: a bit per list entry j > i; with
// coalescence, the first connection in the reference's order whose Weber number exceeds the
// threshold (foam_dynamics.rs:218-232). The connections are observable only after a call, so
// without coalescence this pass runs on a call's last step alone.
//
// The neighbour list holds every pair within range while no bubble has moved skin / 2 since its
// build. The force pass flags a rebuild once a new position is within one step's travel
// (v_max |dt|) of 0.45 skin, so the positions of the next step, which this pass and the next force
// pass read, are still covered.
__global__ void __launch_bounds__(kThreads) connections_kernel(DynArgs a) {
    Ctl *c = a.ctl;
    if (c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t count = 0;
    if (pos < n) {
        const uint32_t i = a.perm[pos];
        const Phys &P = a.P;
        const float4 me = a.pr_out[i];
        const float4 mv = a.vt_out[i];
        const uint32_t m = a.cnt[i], t0 = a.split[i];
        const size_t g0 = a.goff[pos >> 5];
        const uint32_t *col = a.nbr + g0 + (pos & 31);
        uint32_t *fcol = a.cflag + (g0 >> 5) + (pos & 31);
        const float threshold = -me.w * 0.3f;
        bool want = P.coalescence != 0;
        uint32_t word = 0;
        for (uint32_t t = t0; t < m; ++t) {  // the entries j > i
            const uint32_t j = __ldg(col + (size_t)t * 32);
            {
                const float4 o = a.pr_out[j];
                const float overlap = me.w + o.w - len3(me.x - o.x, me.y - o.y, me.z - o.z);
                if (overlap > threshold) {
                    word |= 1u << (t & 31);
                    ++count;
                    if (want) {
                        // BubbleConnection::new's normal, then the Weber number
                        const float dx = o.x - me.x, dy = o.y - me.y, dz = o.z - me.z;
                        const float d = len3(dx, dy, dz);
                        const float nx = dx / d, ny = dy / d, nz = dz / d;
                        const float4 ov = a.vt_out[j];
                        const float rel = (ov.x - mv.x) * nx + (ov.y - mv.y) * ny + (ov.z - mv.z) * nz;
                        const float weber = P.density * (rel * rel) * me.w / P.surface_tension;
                        if (weber > P.coal_threshold) {
                            atomicMin(&c->coal_key, ((unsigned long long)i << 32) | j);
                            want = false;
                        }
                    }
                }
            }
            if ((t & 31) == 31) {
                fcol[(size_t)(t >> 5) * 32] = word;
                word = 0;
            }
        }
        if (m & 31) fcol[(size_t)(m >> 5) * 32] = word;
    }
    for (int o = 16; o; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd(&c->nconn, count);
}

// handle_coalescence's merge (foam.rs:369-405): compacts the cluster without the two bubbles and
// appends the merged one; copies the state unchanged when nothing merges.
__global__ void __launch_bounds__(kThreads) merge_kernel(DynArgs a) {
    Ctl *c = a.ctl;
    if (c->fault != kFaultNone) return;
    const uint32_t n = c->n[a.npar];
    const unsigned long long key = c->coal_key;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (key == kNoPair) {
        if (i < n) {
            a.pr_out[i] = a.pr_in[i];
            a.vt_out[i] = a.vt_in[i];
            a.id_out[i] = a.id_in[i];
        }
        if (i == 0) c->n[a.npar ^ 1] = n;
        return;
    }
    const uint32_t ia = (uint32_t)(key >> 32), ib = (uint32_t)key;
    if (i < n && i != ia && i != ib) {
        const uint32_t d = i - (i > ia) - (i > ib);
        a.pr_out[d] = a.pr_in[i];
        a.vt_out[d] = a.vt_in[i];
        a.id_out[d] = a.id_in[i];
    }
    if (i == 0) {
        const float4 pa = a.pr_in[ia], pb = a.pr_in[ib], va = a.vt_in[ia], vb = a.vt_in[ib];
        const float vol_a = (4.0f / 3.0f) * kPi * (pa.w * (pa.w * pa.w));
        const float vol_b = (4.0f / 3.0f) * kPi * (pb.w * (pb.w * pb.w));
        const float vol_total = vol_a + vol_b;
        const float base = vol_total * 3.0f / (4.0f * kPi);
        const float r = (float)pow((double)base, (double)(1.0f / 3.0f));
        const float area_a = 4.0f * kPi * (pa.w * pa.w), area_b = 4.0f * kPi * (pb.w * pb.w);
        const float t = (va.w * area_a + vb.w * area_b) / (area_a + area_b);
        a.pr_out[n - 2] = make_float4((pa.x * vol_a + pb.x * vol_b) / vol_total, (pa.y * vol_a + pb.y * vol_b) / vol_total,
                                      (pa.z * vol_a + pb.z * vol_b) / vol_total, r);
        a.vt_out[n - 2] = make_float4((va.x * vol_a + vb.x * vol_b) / vol_total, (va.y * vol_a + vb.y * vol_b) / vol_total,
                                      (va.z * vol_a + vb.z * vol_b) / vol_total, t);
        a.id_out[n - 2] = c->next_id;
        c->next_id += 1;
        c->merged_a = a.id_in[ia];
        c->merged_b = a.id_in[ib];
        c->n[a.npar ^ 1] = n - 1;
        c->need_rebuild = 1;
    }
}

// ----------------------------------------------------------------------------- queries
struct ConnArgs {
    const Ctl *ctl;
    uint32_t n;  // count before the merge of the last step
    const uint32_t *split, *inv;
    float surface_tension;
    const float4 *pr, *vt;
    const uint32_t *id;
    const uint32_t *cnt, *goff, *nbr, *cflag;
    uint32_t *per;   // connections per bubble (kept ones)
    uint32_t *off;   // their offsets
    sbs_bubble_connection *out;
    uint32_t cap;
};

__device__ __forceinline__ bool conn_kept(const ConnArgs &a, uint32_t i, uint32_t j) {
    const uint32_t ma = a.ctl->merged_a, mb = a.ctl->merged_b;
    const uint32_t x = a.id[i], y = a.id[j];
    return !(ma != kNone && (x == ma || x == mb || y == ma || y == mb));
}

template <bool kWrite>
__global__ void conn_list_kernel(ConnArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint32_t m = a.cnt[i], pos = a.inv[i];
    const size_t g0 = a.goff[pos >> 5];
    const uint32_t *col = a.nbr + g0 + (pos & 31);
    const uint32_t *fcol = a.cflag + (g0 >> 5) + (pos & 31);
    uint32_t k = 0, o = kWrite ? a.off[i] : 0;
    for (uint32_t t = a.split[i]; t < m; ++t) {
        if (!((fcol[(size_t)(t >> 5) * 32] >> (t & 31)) & 1u)) continue;
        const uint32_t j = col[(size_t)t * 32];
        if (!conn_kept(a, i, j)) continue;
        if (kWrite) {
            if (o < a.cap) {
                // BubbleConnection::new (foam.rs:107-141)
                const float4 pa = a.pr[i], pb = a.pr[j];
                const float ta = a.vt[i].w, tb = a.vt[j].w;
                const float dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
                const float d = len3(dx, dy, dz);
                const float tt = pa.w / (pa.w + pb.w);
                sbs_bubble_connection r;
                r.bubble_a = a.id[i];
                r.bubble_b = a.id[j];
                r.contact_point[0] = pa.x + dx * tt;
                r.contact_point[1] = pa.y + dy * tt;
                r.contact_point[2] = pa.z + dz * tt;
                r.contact_normal[0] = dx / d;
                r.contact_normal[1] = dy / d;
                r.contact_normal[2] = dz / d;
                const float p_a = 4.0f * a.surface_tension / pa.w, p_b = 4.0f * a.surface_tension / pb.w;
                const float dp = p_a - p_b;
                r.wall_curvature_radius = fabsf(dp) > 1e-6f ? 2.0f * a.surface_tension / dp : INFINITY;
                r.wall_thickness_nm = (ta + tb) / 2.0f * 0.8f;
                a.out[o] = r;
            }
            ++o;
        } else {
            ++k;
        }
    }
    if (!kWrite) a.per[i] = k;
}

__global__ void unpack_kernel(uint32_t n, const float4 *pr, const float4 *vt, const uint32_t *id, float *pos, float *vel,
                              float *radius, float *thick, uint32_t *ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pr[i], v = vt[i];
    if (pos) {
        pos[3 * (size_t)i] = p.x;
        pos[3 * (size_t)i + 1] = p.y;
        pos[3 * (size_t)i + 2] = p.z;
    }
    if (vel) {
        vel[3 * (size_t)i] = v.x;
        vel[3 * (size_t)i + 1] = v.y;
        vel[3 * (size_t)i + 2] = v.z;
    }
    if (radius) radius[i] = p.w;
    if (thick) thick[i] = v.w;
    if (ids) ids[i] = id[i];
}

__global__ void pack_kernel(uint32_t n, float4 *pr, float4 *vt, const float *pos, const float *vel,
                            const float *radius, const float *thick) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pr[i], v = vt[i];
    if (pos) p = make_float4(pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2], p.w);
    if (radius) p.w = radius[i];
    if (vel) v = make_float4(vel[3 * (size_t)i], vel[3 * (size_t)i + 1], vel[3 * (size_t)i + 2], v.w);
    if (thick) v.w = thick[i];
    pr[i] = p;
    vt[i] = v;
}

__global__ void set_thickness_kernel(uint32_t n, float4 *vt, const float *thick) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) vt[i].w = thick[i];
}

unsigned blocks(size_t n, int t = kThreads) { return (unsigned)std::max<size_t>(1, (n + t - 1) / t); }

}  // namespace
}  // namespace sbs

using namespace sbs;

struct sbs_foam_sim {
    uint32_t n_cap = 0;
    uint32_t mask = 0;
    sbs_foam_physics phys{};
    cudaStream_t stream = nullptr;
    Ctl *ctl = nullptr;
    Bufs b{};
    int cur = 0, npar = 0, conn_buf = 0, conn_npar = 0;
    bool list_invalid = true, stepped = false;
    bool conn_cached = false;  // connections of the last step kept on the host (see sbs_foam_sim_forces)
    std::vector<sbs_bubble_connection> conn_cache;
    float list_skin = -1.0f;  // skin of the current neighbour list
    float4 *p0 = nullptr;
    int4 *cellc = nullptr;
    uint32_t *bcount = nullptr, *bstart = nullptr, *bitems = nullptr, *bkey = nullptr, *brank = nullptr;
    float4 *spr = nullptr;
    unsigned long long *skey = nullptr;
    int list_blocks = 1;  // grid of the count / walk / sort passes (a few blocks per SM, grid-stride)
    uint32_t *cnt = nullptr, *split = nullptr, *gcap = nullptr, *goff = nullptr;
    uint32_t *perm = nullptr, *inv = nullptr, *mhist = nullptr, *mstart = nullptr;
    uint32_t *nbr = nullptr, *cflag = nullptr;
    size_t nbr_cap = 0;
    float rmax0 = 0.0f;
};

namespace {

Phys phys_of(const sbs_foam_physics &p) {
    Phys P;
    P.surface_tension = p.surface_tension;
    P.viscosity = p.viscosity;
    P.density = p.density;
    P.gx = p.gravity[0];
    P.gy = p.gravity[1];
    P.gz = p.gravity[2];
    P.vdw = p.van_der_waals_strength;
    P.stiffness = p.repulsion_stiffness;
    P.damping = p.damping;
    P.coal_threshold = p.coalescence_threshold;
    P.coalescence = p.coalescence_enabled ? 1 : 0;
    return P;
}

int check_physics(const sbs_foam_physics *p) {
    SBS_CHECK_ARG(p != nullptr, "physics is null");
    const float v[] = {p->surface_tension, p->viscosity, p->density, p->gravity[0], p->gravity[1], p->gravity[2],
                       p->van_der_waals_strength, p->repulsion_stiffness, p->damping, p->coalescence_threshold};
    for (float x : v) SBS_CHECK_ARG(std::isfinite(x), "physics parameters must be finite");
    return SBS_OK;
}

ListArgs list_args(sbs_foam_sim *s) {
    ListArgs a;
    a.ctl = s->ctl;
    a.npar = s->npar;
    a.pr = s->b.pr[s->cur];
    a.p0 = s->p0;
    a.cellc = s->cellc;
    a.bcount = s->bcount;
    a.bstart = s->bstart;
    a.bitems = s->bitems;
    a.spr = s->spr;
    a.skey = s->skey;
    a.bkey = s->bkey;
    a.brank = s->brank;
    a.mask = s->mask;
    a.cnt = s->cnt;
    a.split = s->split;
    a.gcap = s->gcap;
    a.perm = s->perm;
    a.inv = s->inv;
    a.mhist = s->mhist;
    a.mstart = s->mstart;
    a.goff = s->goff;
    a.nbr = s->nbr;
    a.nbr_cap = s->nbr_cap;
    return a;
}

// Skin of the neighbour list: about 80 steps of travel at the speed limit, between 8 % and 20 % of
// the largest interaction range 6 r_max (the extra candidates cost a squared-distance test each),
// and never below 2.5 steps of travel.
float skin_for(const sbs_foam_sim *s, float dt) {
    const float range = 6.0f * s->rmax0;
    const float travel = kMaxSpeed * std::fabs(dt);
    const float want = std::min(std::max(2.02f * travel * 80.0f, 0.08f * range), 0.2f * range);
    return std::max(want, 2.5f * travel);
}

// Squared displacement beyond which the connection pass flags a rebuild (< 0: every step).
float flag_sq_for(float skin, float dt) {
    const float h = 0.45f * skin - 1.01f * kMaxSpeed * std::fabs(dt);
    return h > 0.0f ? h * h : -1.0f;
}

void enqueue_list(sbs_foam_sim *s, bool forced, float skin) {
    ListArgs a = list_args(s);
    s->list_skin = skin;
    cudaMemsetAsync(s->bcount, 0, sizeof(uint32_t) * (s->mask + 1), s->stream);
    cudaMemsetAsync(s->mhist, 0, sizeof(uint32_t) * (kMaxCand + 1), s->stream);
    list_begin_kernel<<<1, 1024, 0, s->stream>>>(a, forced ? 1 : 0, skin);
    list_bin_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
    scan_kernel<<<1, 1024, 0, s->stream>>>(s->bcount, s->bstart, s->mask + 1, 0, a);
    list_scatter_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
    list_count_kernel<<<s->list_blocks, kListWarps * 32, 0, s->stream>>>(a);
    scan_kernel<<<1, 1024, 0, s->stream>>>(s->mhist, s->mstart, kMaxCand + 1, 0, a);
    list_order_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
    list_gcap_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
    scan_kernel<<<1, 1024, 0, s->stream>>>(s->gcap, s->goff, 0, 1, a);
    list_walk_kernel<<<s->list_blocks, kListWarps * 32, 0, s->stream>>>(a);
    list_sort_kernel<<<s->list_blocks, kListWarps * 32, 0, s->stream>>>(a);
}

DynArgs dyn_args(sbs_foam_sim *s, float dt, int in, int out) {
    DynArgs a;
    a.ctl = s->ctl;
    a.npar = s->npar;
    a.P = phys_of(s->phys);
    a.dt = dt;
    a.pr_in = s->b.pr[in];
    a.vt_in = s->b.vt[in];
    a.id_in = s->b.id[in];
    a.pr_out = s->b.pr[out];
    a.vt_out = s->b.vt[out];
    a.id_out = s->b.id[out];
    a.force_out = nullptr;
    a.cnt = s->cnt;
    a.split = s->split;
    a.perm = s->perm;
    a.goff = s->goff;
    a.nbr = s->nbr;
    a.cflag = s->cflag;
    a.p0 = s->p0;
    a.flag_sq = flag_sq_for(s->list_skin, dt);
    return a;
}

// Lanes per bubble of the force pass: enough threads to fill the GPU's SMs for small foams.
void launch_forces(sbs_foam_sim *s, const DynArgs &a) {
    const uint32_t n = s->n_cap;
    if (n >= 131072)
        forces_kernel<1><<<blocks(n), kThreads, 0, s->stream>>>(a);
    else if (n >= 32768)
        forces_kernel<4><<<blocks((size_t)n * 4), kThreads, 0, s->stream>>>(a);
    else
        forces_kernel<16><<<blocks((size_t)n * 16), kThreads, 0, s->stream>>>(a);
}

void free_list(sbs_foam_sim *s) {
    cudaFree(s->nbr);
    cudaFree(s->cflag);
    s->nbr = s->cflag = nullptr;
    s->nbr_cap = 0;
}

int alloc_list(sbs_foam_sim *s, size_t entries) {
    free_list(s);
    entries = (entries + 1023) & ~(size_t)1023;
    SBS_CUDA_TRY(cudaMalloc(&s->nbr, sizeof(uint32_t) * entries));
    SBS_CUDA_TRY(cudaMalloc(&s->cflag, sizeof(uint32_t) * (entries / 32)));
    s->nbr_cap = entries;
    return SBS_OK;
}

int read_ctl(sbs_foam_sim *s, Ctl *h) {
    SBS_CUDA_TRY(cudaMemcpyAsync(h, s->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

// Builds the neighbour list for the current state, growing its storage as needed.
int rebuild_now(sbs_foam_sim *s, float skin) {
    for (int attempt = 0; attempt < 3; ++attempt) {
        enqueue_list(s, true, skin);
        SBS_CUDA_TRY(cudaGetLastError());
        Ctl h;
        int rc = read_ctl(s, &h);
        if (rc) return rc;
        if (h.fault == kFaultDense)
            return set_error(SBS_E_INVALID,
                             "foam too dense: bubble %u has %u neighbours within 3 (r_a + r_b) + skin (limit %d)",
                             h.dense_bubble, h.dense_count, kMaxCand);
        if (h.fault == kFaultWalk) return set_error(SBS_E_STATE, "foam neighbour list: walk and count passes disagree");
        if (h.fault == kFaultNone) {
            s->list_invalid = false;
            return SBS_OK;
        }
        SBS_CUDA_TRY(cudaMemsetAsync(&s->ctl->fault, 0, sizeof(uint32_t), s->stream));
        if ((rc = alloc_list(s, (size_t)h.list_total + h.list_total / 2 + 1024))) return rc;
    }
    return set_error(SBS_E_CUDA, "foam neighbour list: could not size the list");
}

int current_n(sbs_foam_sim *s, uint32_t *n) {
    SBS_CUDA_TRY(cudaMemcpyAsync(n, &s->ctl->n[s->npar], sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

}  // namespace

extern "C" {

int sbs_foam_physics_default(sbs_foam_physics *out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->surface_tension = 0.025f;
    out->viscosity = 0.001f;
    out->density = 1000.0f;
    out->gravity[1] = -9.81f;
    out->van_der_waals_strength = 0.001f;
    out->repulsion_stiffness = 5.0f;
    out->damping = 0.8f;
    out->coalescence_enabled = 0;
    out->coalescence_threshold = 0.5f;
    return SBS_OK;
}

int sbs_foam_sim_destroy(sbs_foam_sim *s) {
    if (!s) return SBS_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (int k = 0; k < 2; ++k) {
        cudaFree(s->b.pr[k]);
        cudaFree(s->b.vt[k]);
        cudaFree(s->b.id[k]);
    }
    cudaFree(s->ctl);
    cudaFree(s->p0);
    cudaFree(s->cellc);
    cudaFree(s->bcount);
    cudaFree(s->bstart);
    cudaFree(s->bitems);
    cudaFree(s->spr);
    cudaFree(s->skey);
    cudaFree(s->bkey);
    cudaFree(s->brank);
    cudaFree(s->cnt);
    cudaFree(s->split);
    cudaFree(s->perm);
    cudaFree(s->inv);
    cudaFree(s->mhist);
    cudaFree(s->mstart);
    cudaFree(s->gcap);
    cudaFree(s->goff);
    free_list(s);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SBS_OK;
}

int sbs_foam_sim_create(uint32_t n, const float *position, const float *radius, const float *thickness_nm,
                        const sbs_foam_physics *p, sbs_foam_sim **out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    SBS_CHECK_ARG(n >= 1 && n <= (1u << 26), "bubble count %u out of range (1 .. 2^26)", n);
    SBS_CHECK_ARG(position != nullptr && radius != nullptr, "null position or radius");
    int rc = check_physics(p);
    if (rc) return rc;
    float rmax = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        SBS_CHECK_ARG(radius[i] > 0.0f && std::isfinite(radius[i]), "bubble %u: radius must be > 0", i);
        for (int d = 0; d < 3; ++d)
            SBS_CHECK_ARG(std::isfinite(position[3 * (size_t)i + d]), "bubble %u: position must be finite", i);
        SBS_CHECK_ARG(!thickness_nm || std::isfinite(thickness_nm[i]), "bubble %u: thickness must be finite", i);
        rmax = std::max(rmax, radius[i]);
    }
    if ((rc = require_device())) return rc;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return set_error(SBS_E_CUDA, "foam dynamics: no device attributes");
    sbs_foam_sim *s = new sbs_foam_sim();
    s->n_cap = n;
    s->list_blocks = (int)std::max<uint32_t>(1, std::min<uint32_t>((n + kListWarps - 1) / kListWarps, (uint32_t)sms * 16));
    s->phys = *p;
    s->rmax0 = rmax;
    uint32_t M = 1024;
    while (M < n) M <<= 1;
    s->mask = M - 1;
    const uint32_t groups = (n + 31) / 32;
    auto fail = [&](cudaError_t e) {
        sbs_foam_sim_destroy(s);
        return set_error(SBS_E_CUDA, "foam dynamics: allocation failed: %s", cudaGetErrorString(e));
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        if (e == cudaSuccess) e = cudaMalloc(&s->b.pr[k], sizeof(float4) * n);
        if (e == cudaSuccess) e = cudaMalloc(&s->b.vt[k], sizeof(float4) * n);
        if (e == cudaSuccess) e = cudaMalloc(&s->b.id[k], sizeof(uint32_t) * n);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMalloc(&s->p0, sizeof(float4) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->cellc, sizeof(int4) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->bcount, sizeof(uint32_t) * M);
    if (e == cudaSuccess) e = cudaMalloc(&s->bstart, sizeof(uint32_t) * (M + 1));
    if (e == cudaSuccess) e = cudaMalloc(&s->bitems, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->spr, sizeof(float4) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->skey, sizeof(unsigned long long) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->bkey, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->brank, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->cnt, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->split, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->perm, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->inv, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s->mhist, sizeof(uint32_t) * (kMaxCand + 1));
    if (e == cudaSuccess) e = cudaMalloc(&s->mstart, sizeof(uint32_t) * (kMaxCand + 2));
    if (e == cudaSuccess) e = cudaMalloc(&s->gcap, sizeof(uint32_t) * groups);
    if (e == cudaSuccess) e = cudaMalloc(&s->goff, sizeof(uint32_t) * (groups + 1));
    if (e != cudaSuccess) return fail(e);
    std::vector<float4> pr(n), vt(n);
    std::vector<uint32_t> ids(n);
    for (uint32_t i = 0; i < n; ++i) {
        pr[i] = make_float4(position[3 * (size_t)i], position[3 * (size_t)i + 1], position[3 * (size_t)i + 2], radius[i]);
        vt[i] = make_float4(0.0f, 0.0f, 0.0f, thickness_nm ? thickness_nm[i] : 500.0f);  // Bubble::new
        ids[i] = i;
    }
    Ctl c;
    std::memset(&c, 0, sizeof(c));
    c.n[0] = c.n[1] = n;
    c.next_id = n;
    c.coal_key = kNoPair;
    c.merged_a = c.merged_b = kNone;
    e = cudaMemcpyAsync(s->b.pr[0], pr.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->b.vt[0], vt.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->b.id[0], ids.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->ctl, &c, sizeof(c), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail(e);
    *out = s;
    return SBS_OK;
}

int sbs_foam_sim_set_physics(sbs_foam_sim *s, const sbs_foam_physics *p) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr, "handle is null");
    int rc = check_physics(p);
    if (rc) return rc;
    s->phys = *p;
    return SBS_OK;
}

int sbs_foam_sim_step(sbs_foam_sim *s, float dt, uint32_t steps) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr, "handle is null");
    SBS_CHECK_ARG(std::isfinite(dt), "dt must be finite");
    if (steps == 0) return SBS_OK;
    const bool coal = s->phys.coalescence_enabled != 0;
    const float skin = skin_for(s, dt);
    if (skin != s->list_skin) s->list_invalid = true;  // a new dt: a list built for this step size
    s->conn_cached = false;
    uint32_t done = 0;
    while (done < steps) {
        int rc;
        if (s->list_invalid && (rc = rebuild_now(s, skin))) return rc;
        const int cur0 = s->cur, npar0 = s->npar;
        SBS_CUDA_TRY(cudaMemsetAsync(&s->ctl->steps_done, 0, sizeof(uint32_t), s->stream));
        for (uint32_t k = done; k < steps; ++k) {
            enqueue_list(s, false, skin);
            DynArgs a = dyn_args(s, dt, s->cur, s->cur ^ 1);
            launch_forces(s, a);
            if (coal || k + 1 == steps) connections_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
            s->conn_buf = s->cur ^ 1;
            s->conn_npar = s->npar;
            if (coal) {
                DynArgs m = dyn_args(s, dt, s->cur ^ 1, s->cur);
                merge_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(m);
                s->npar ^= 1;
            } else {
                s->cur ^= 1;
            }
        }
        SBS_CUDA_TRY(cudaGetLastError());
        Ctl h;
        if ((rc = read_ctl(s, &h))) return rc;
        s->stepped = true;
        if (h.fault == kFaultNone) break;
        if (h.fault == kFaultWalk) return set_error(SBS_E_STATE, "foam neighbour list: walk and count passes disagree");
        // The list outgrew its storage at a rebuild: the steps from there on did nothing. Restore
        // the buffer parities of the last completed step, grow the list and continue.
        done += h.steps_done;
        if (coal) {
            s->cur = cur0;
            s->npar = npar0 ^ (int)(h.steps_done & 1);
            s->conn_buf = cur0 ^ 1;
            s->conn_npar = s->npar ^ 1;
        } else {
            s->cur = cur0 ^ (int)(h.steps_done & 1);
            s->conn_buf = s->cur;
            s->conn_npar = s->npar;
        }
        if (h.fault == kFaultDense)
            return set_error(SBS_E_INVALID,
                             "foam too dense: bubble %u has %u neighbours within 3 (r_a + r_b) + skin (limit %d)",
                             h.dense_bubble, h.dense_count, kMaxCand);
        SBS_CUDA_TRY(cudaMemsetAsync(&s->ctl->fault, 0, sizeof(uint32_t), s->stream));
        if ((rc = alloc_list(s, (size_t)h.list_total + h.list_total / 2 + 1024))) return rc;
        s->list_invalid = true;
    }
    return SBS_OK;
}

int sbs_foam_sim_counts(sbs_foam_sim *s, uint32_t *bubbles, uint32_t *connections) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr, "handle is null");
    Ctl h;
    int rc = read_ctl(s, &h);
    if (rc) return rc;
    if (bubbles) *bubbles = h.n[s->npar];
    if (connections) {
        if (!s->stepped) {
            uint32_t c = 0;
            if ((rc = sbs_foam_sim_connections(s, nullptr, 0, &c))) return rc;
            *connections = c;
        } else if (h.merged_a == kNone) {
            *connections = h.nconn;
        } else {
            uint32_t c = 0;
            if ((rc = sbs_foam_sim_connections(s, nullptr, 0, &c))) return rc;
            *connections = c;
        }
    }
    return SBS_OK;
}

int sbs_foam_sim_get_state(sbs_foam_sim *s, float *position, float *velocity, float *radius, float *thickness_nm,
                           uint32_t *ids, int mem) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr, "handle is null");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    uint32_t n = 0;
    int rc = current_n(s, &n);
    if (rc) return rc;
    const int c = s->cur;
    if (mem == SBS_MEM_DEVICE) {
        unpack_kernel<<<blocks(n), kThreads, 0, s->stream>>>(n, s->b.pr[c], s->b.vt[c], s->b.id[c], position, velocity,
                                                             radius, thickness_nm, ids);
        SBS_CUDA_TRY(cudaGetLastError());
        SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        return SBS_OK;
    }
    // unpacked on the device into one scratch block, then copied straight into the caller's arrays
    float *dev[4] = {nullptr, nullptr, nullptr, nullptr};
    uint32_t *dids = nullptr;
    float *host[4] = {position, velocity, radius, thickness_nm};
    const size_t len[4] = {3 * (size_t)n, 3 * (size_t)n, n, n};
    size_t total = ids ? n : 0;
    for (int k = 0; k < 4; ++k) total += host[k] ? len[k] : 0;
    if (total == 0) return SBS_OK;
    char *base = nullptr;
    SBS_CUDA_TRY(scratch_alloc((void **)&base, sizeof(float) * total + 64, s->stream));
    size_t o = 0;
    for (int k = 0; k < 4; ++k)
        if (host[k]) {
            dev[k] = (float *)base + o;
            o += len[k];
        }
    if (ids) dids = (uint32_t *)((float *)base + o);
    unpack_kernel<<<blocks(n), kThreads, 0, s->stream>>>(n, s->b.pr[c], s->b.vt[c], s->b.id[c], dev[0], dev[1], dev[2],
                                                         dev[3], dids);
    cudaError_t e = cudaGetLastError();
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (host[k]) e = cudaMemcpyAsync(host[k], dev[k], sizeof(float) * len[k], cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && ids) e = cudaMemcpyAsync(ids, dids, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream);
    cudaFreeAsync(base, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "foam get_state: %s", cudaGetErrorString(e));
    return SBS_OK;
}

int sbs_foam_sim_set_state(sbs_foam_sim *s, const float *position, const float *velocity, const float *radius,
                           const float *thickness_nm, int mem) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr, "handle is null");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    uint32_t n = 0;
    int rc = current_n(s, &n);
    if (rc) return rc;
    if (mem == SBS_MEM_HOST && radius)
        for (uint32_t i = 0; i < n; ++i)
            SBS_CHECK_ARG(radius[i] > 0.0f && std::isfinite(radius[i]), "bubble %u: radius must be > 0", i);
    const float *src[4] = {position, velocity, radius, thickness_nm};
    const size_t len[4] = {3 * (size_t)n, 3 * (size_t)n, n, n};
    float *dev[4] = {nullptr, nullptr, nullptr, nullptr};
    char *base = nullptr;
    if (mem == SBS_MEM_HOST) {
        size_t total = 0;
        for (int k = 0; k < 4; ++k) total += src[k] ? len[k] : 0;
        SBS_CUDA_TRY(scratch_alloc((void **)&base, sizeof(float) * total + 64, s->stream));
        size_t o = 0;
        for (int k = 0; k < 4; ++k)
            if (src[k]) {
                dev[k] = (float *)base + o;
                cudaMemcpyAsync(dev[k], src[k], sizeof(float) * len[k], cudaMemcpyHostToDevice, s->stream);
                o += len[k];
            }
    } else {
        for (int k = 0; k < 4; ++k) dev[k] = const_cast<float *>(src[k]);
    }
    pack_kernel<<<blocks(n), kThreads, 0, s->stream>>>(n, s->b.pr[s->cur], s->b.vt[s->cur], dev[0], dev[1], dev[2],
                                                       dev[3]);
    cudaError_t e = cudaGetLastError();
    if (base) cudaFreeAsync(base, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "foam set_state: %s", cudaGetErrorString(e));
    if (radius) {
        std::vector<float4> pr(n);
        SBS_CUDA_TRY(cudaMemcpy(pr.data(), s->b.pr[s->cur], sizeof(float4) * n, cudaMemcpyDeviceToHost));
        float m = 0.0f;
        for (const float4 &q : pr) m = std::max(m, q.w);
        s->rmax0 = m;
    }
    s->list_invalid = true;
    s->stepped = false;
    s->conn_cached = false;
    return SBS_OK;
}

int sbs_foam_sim_forces(sbs_foam_sim *s, float *forces, int mem) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr && forces != nullptr, "null argument");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    int rc;
    if (s->list_invalid) {
        if ((rc = rebuild_now(s, skin_for(s, 0.0f)))) return rc;
    } else {
        Ctl h;
        if ((rc = read_ctl(s, &h))) return rc;
        if (h.need_rebuild) {
            // the rebuild overwrites the list that the last step's connections are read from: keep
            // them on the host first
            if (s->stepped && !s->conn_cached) {
                uint32_t count = 0;
                if ((rc = sbs_foam_sim_connections(s, nullptr, 0, &count))) return rc;
                std::vector<sbs_bubble_connection> keep(count);
                if (count && (rc = sbs_foam_sim_connections(s, keep.data(), count, &count))) return rc;
                s->conn_cache.swap(keep);
                s->conn_cached = true;
            }
            enqueue_list(s, false, s->list_skin);
        }
    }
    uint32_t n = 0;
    if ((rc = current_n(s, &n))) return rc;
    float *dout = forces;
    if (mem == SBS_MEM_HOST) SBS_CUDA_TRY(scratch_alloc((void **)&dout, sizeof(float) * 3 * n, s->stream));
    DynArgs a = dyn_args(s, 0.0f, s->cur, s->cur ^ 1);
    a.force_out = dout;
    launch_forces(s, a);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && mem == SBS_MEM_HOST)
        e = cudaMemcpyAsync(forces, dout, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s->stream);
    if (mem == SBS_MEM_HOST) cudaFreeAsync(dout, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "foam forces: %s", cudaGetErrorString(e));
    return SBS_OK;
}

int sbs_foam_sim_connections(sbs_foam_sim *s, sbs_bubble_connection *out, uint32_t capacity, uint32_t *count) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr && count != nullptr, "null argument");
    SBS_CHECK_ARG(out != nullptr || capacity == 0, "null output with capacity %u", capacity);
    int rc;
    if (s->stepped && s->conn_cached) {
        *count = (uint32_t)s->conn_cache.size();
        const size_t k = std::min<size_t>(capacity, s->conn_cache.size());
        if (k) std::memcpy(out, s->conn_cache.data(), k * sizeof(sbs_bubble_connection));
        return SBS_OK;
    }
    if (!s->stepped) {
        // before any step: BubbleCluster::update_connections of the initial state (FoamGenerator::
        // generate and create_default_cluster end with it), flags from a connection pass alone
        if (s->list_invalid && (rc = rebuild_now(s, skin_for(s, 0.0f)))) return rc;
        SBS_CUDA_TRY(cudaMemsetAsync(&s->ctl->merged_a, 0xff, 2 * sizeof(uint32_t), s->stream));
        DynArgs a = dyn_args(s, 0.0f, s->cur, s->cur);
        a.P.coalescence = 0;
        connections_kernel<<<blocks(s->n_cap), kThreads, 0, s->stream>>>(a);
        SBS_CUDA_TRY(cudaGetLastError());
        s->conn_buf = s->cur;
        s->conn_npar = s->npar;
    }
    uint32_t n = 0;
    SBS_CUDA_TRY(cudaMemcpyAsync(&n, &s->ctl->n[s->conn_npar], sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    uint32_t *per = nullptr;
    SBS_CUDA_TRY(scratch_alloc((void **)&per, sizeof(uint32_t) * (2 * (size_t)n + 2), s->stream));
    uint32_t *off = per + n + 1;
    sbs_bubble_connection *dout = nullptr;
    ConnArgs a;
    a.ctl = s->ctl;
    a.n = n;
    a.surface_tension = s->phys.surface_tension;
    a.pr = s->b.pr[s->conn_buf];
    a.vt = s->b.vt[s->conn_buf];
    a.id = s->b.id[s->conn_buf];
    a.cnt = s->cnt;
    a.split = s->split;
    a.inv = s->inv;
    a.goff = s->goff;
    a.nbr = s->nbr;
    a.cflag = s->cflag;
    a.per = per;
    a.off = off;
    a.out = nullptr;
    a.cap = 0;
    conn_list_kernel<false><<<blocks(n), kThreads, 0, s->stream>>>(a);
    // the host scans the per-bubble counts (a query, not a step)
    std::vector<uint32_t> hper(n), hoff(n + 1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hper.data(), per, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(per, s->stream);
        return set_error(SBS_E_CUDA, "foam connections: %s", cudaGetErrorString(e));
    }
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        hoff[i] = (uint32_t)total;
        total += hper[i];
    }
    hoff[n] = (uint32_t)total;
    *count = (uint32_t)total;
    const uint32_t want = (uint32_t)std::min<uint64_t>(total, capacity);
    if (want > 0) {
        e = cudaMemcpyAsync(off, hoff.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = scratch_alloc((void **)&dout, sizeof(sbs_bubble_connection) * want, s->stream);
        if (e == cudaSuccess) {
            a.out = dout;
            a.cap = want;
            conn_list_kernel<true><<<blocks(n), kThreads, 0, s->stream>>>(a);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out, dout, sizeof(sbs_bubble_connection) * want, cudaMemcpyDeviceToHost, s->stream);
        if (dout) cudaFreeAsync(dout, s->stream);
    }
    cudaFreeAsync(per, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "foam connections: %s", cudaGetErrorString(e));
    return SBS_OK;
}

int sbs_foam_sim_couple_thickness(sbs_foam_sim *s, sbs_foam *batch) {
    clear_error();
    SBS_CHECK_ARG(s != nullptr && batch != nullptr, "null argument");
    uint32_t n = 0;
    int rc = current_n(s, &n);
    if (rc) return rc;
    float *mean = nullptr;
    SBS_CUDA_TRY(cudaMalloc(&mean, sizeof(float) * n));
    uint32_t nb = 0;
    rc = foam_mean_thickness_nm(batch, mean, n, &nb);
    if (rc == SBS_OK && nb != n)
        rc = set_error(SBS_E_INVALID, "the batch has %u bubbles, the cluster %u", nb, n);
    if (rc == SBS_OK) {
        set_thickness_kernel<<<blocks(n), kThreads, 0, s->stream>>>(n, s->b.vt[s->cur], mean);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) rc = set_error(SBS_E_CUDA, "foam coupling: %s", cudaGetErrorString(e));
    }
    cudaFree(mean);
    return rc;
}

}  // extern "C"

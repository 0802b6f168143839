// DOF-object numbering and boundary detection on the GPU.
//
// The same rules as the host pipeline in isl_host.cpp, which follows
// base/dof/generateDoFIndicesFromFaces.hpp:169-298 and
// base/mesh/createBoundaryFromUnstructured.hpp:51-109:
//  * n-faces (vertices, edges, faces) of the elements are identified by their
//    sorted vertex ids; the occurrences of one n-face form a group, and the
//    group's first occurrence in element-major slot order (slot = element *
//    faces per element + local face) carries it;
//  * numbering: per instance, level by level (vertices, edges, faces, cell),
//    every first occurrence takes the next `stride` ids in slot order and the
//    other occurrences copy them; cell DOFs take ids in element order;
//  * boundary: faces of dimension dim - 1 that occur once, listed in the
//    lexicographic order of their sorted vertex ids.
//
// GPU form: keys are packed vertex ids, slots are ordered by a stable LSD radix
// sort of (key, slot) (two passes for three or four ids); group heads come from
// adjacent key comparisons and group starts from a max-scan; first visits are
// ranked by an exclusive scan in slot order.  Everything is integer work, so
// the results are identical to the host's bit for bit.
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "isl_internal.h"

namespace isl {

namespace {

constexpr int TB = 256;

inline unsigned nblocks(long long n) { return (unsigned)std::max<long long>(1, (n + TB - 1) / TB); }

int bits_needed(uint64_t v) {
    int b = 1;
    while (b < 63 && (1ull << b) <= v) ++b;
    return b;
}

// packed keys of every (element, face) slot: hi = the two smallest sorted
// vertex ids (one id when the face has one vertex), lo = the other one or two
struct KeyTab {
    int nfc, w;
    int v[12][4];
};

__global__ void k_face_keys(int64_t E, KeyTab t, int nb, const int32_t* __restrict__ conn, uint64_t* __restrict__ hi,
                            uint64_t* __restrict__ lo, int32_t* __restrict__ slot) {
    const int64_t n = E * t.nfc;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = s / t.nfc;
        const int f = (int)(s % t.nfc);
        uint64_t k[4] = {0, 0, 0, 0};
        for (int i = 0; i < t.w; ++i) {
            const uint64_t x = (uint32_t)conn[(int64_t)t.v[f][i] * E + e];
            int j = i;
            while (j > 0 && k[j - 1] > x) { k[j] = k[j - 1]; --j; }
            k[j] = x;
        }
        if (t.w == 1) { hi[s] = k[0]; lo[s] = 0; }
        else if (t.w == 2) { hi[s] = (k[0] << nb) | k[1]; lo[s] = 0; }
        else if (t.w == 3) { hi[s] = (k[0] << nb) | k[1]; lo[s] = k[2]; }
        else { hi[s] = (k[0] << nb) | k[1]; lo[s] = (k[2] << nb) | k[3]; }
        slot[s] = (int32_t)s;
    }
}

__global__ void k_gather_key(int64_t n, const int32_t* __restrict__ ord, const uint64_t* __restrict__ key,
                             uint64_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = key[ord[i]];
}

// gs[i] = i at a group head, 0 elsewhere (max-scanned into group starts);
// head[i] = 1 at a group head
__global__ void k_heads(int64_t n, const uint64_t* __restrict__ hs, const uint64_t* __restrict__ lo,
                        const int32_t* __restrict__ ord, int32_t* __restrict__ gs, uint8_t* __restrict__ head) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool h = i == 0 || hs[i] != hs[i - 1] || lo[ord[i]] != lo[ord[i - 1]];
        gs[i] = h ? (int32_t)i : 0;
        head[i] = h ? 1 : 0;
    }
}

// first[slot] = smallest slot of the slot's group; flag[slot] = 1 at first visits
__global__ void k_first(int64_t n, const int32_t* __restrict__ ord, const int32_t* __restrict__ gstart,
                        int32_t* __restrict__ first, int32_t* __restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = ord[i], s0 = ord[gstart[i]];
        first[s] = s0;
        flag[s] = (s == s0) ? 1 : 0;
    }
}

// 1 where the group has one member
__global__ void k_single(int64_t n, const uint8_t* __restrict__ head, uint8_t* __restrict__ single) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        single[i] = (head[i] && (i + 1 == n || head[i + 1])) ? 1 : 0;
}

__device__ inline int instance_of(int64_t e, const int64_t* __restrict__ eoff, int ninst) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (eoff[mid] <= e) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ids of the shared n-faces of one level
__global__ void k_assign(int64_t E, int nfc, int stride, int begin, const int32_t* __restrict__ first,
                         const int32_t* __restrict__ rank, const int64_t* __restrict__ eoff, int ninst,
                         const int64_t* __restrict__ base, int32_t* __restrict__ edof) {
    const int64_t n = E * nfc;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = s / nfc;
        const int f = (int)(s % nfc);
        const int k = instance_of(e, eoff, ninst);
        const int64_t id0 = base[k] + (int64_t)(rank[first[s]] - rank[eoff[k] * nfc]) * stride;
        for (int d = 0; d < stride; ++d) edof[(int64_t)(begin + f * stride + d) * E + e] = (int32_t)(id0 + d);
    }
}

// ids of the cell interior DOFs: element order within the instance
__global__ void k_assign_cell(int64_t E, int per_elem, int begin, const int64_t* __restrict__ eoff, int ninst,
                              const int64_t* __restrict__ base, int32_t* __restrict__ edof) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int k = instance_of(e, eoff, ninst);
        const int64_t id0 = base[k] + (e - eoff[k]) * per_elem;
        for (int d = 0; d < per_elem; ++d) edof[(int64_t)(begin + d) * E + e] = (int32_t)(id0 + d);
    }
}

// instance boundaries of the rank array: rank at slot eoff[k] * nfc
__global__ void k_rank_at(int ninst, const int64_t* __restrict__ eoff, int nfc, const int32_t* __restrict__ rank,
                          int32_t* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k <= ninst) out[k] = rank[eoff[k] * nfc];
}

// SoA [nf][E] -> AoS [E][nf]
__global__ void k_transpose(int64_t E, int nf, const int32_t* __restrict__ soa, int32_t* __restrict__ aos) {
    const int64_t n = E * nf;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / nf;
        const int f = (int)(i % nf);
        aos[i] = soa[(int64_t)f * E + e];
    }
}

KeyTab make_tab(const DeviceLevel& lv) {
    KeyTab t;
    t.nfc = lv.nfc;
    t.w = lv.w;
    for (int f = 0; f < 12; ++f)
        for (int i = 0; i < 4; ++i) t.v[f][i] = (f < lv.nfc && i < lv.w) ? lv.v[f][i] : 0;
    return t;
}

struct MaxOp {
    __device__ int32_t operator()(int32_t a, int32_t b) const { return a > b ? a : b; }
};

// Groups of one level: ord (slots in (key, slot) order), head flags, first
// occurrence and first-visit flags per slot.
struct Groups {
    DBuf<int32_t> ord, first, flag;
    DBuf<uint8_t> head;
};

int group_level(isl_ctx* c, const DeviceLevel& lv, Groups& g, bool need_first) {
    cudaStream_t st = c->stream;
    const int64_t E = c->nelem, n = E * lv.nfc;
    const int nb = bits_needed((uint64_t)std::max<int64_t>(1, c->nnodes - 1));
    const KeyTab t = make_tab(lv);
    DBuf<uint64_t> hi, lo, kout, hi2;
    DBuf<int32_t> slot, ord1, gs;
    ISL_CHECK_CUDA(c, hi.alloc(n));
    ISL_CHECK_CUDA(c, lo.alloc(n));
    ISL_CHECK_CUDA(c, kout.alloc(n));
    ISL_CHECK_CUDA(c, slot.alloc(n));
    ISL_CHECK_CUDA(c, g.ord.alloc(n));
    const unsigned gr = std::min<unsigned>(nblocks(n), (unsigned)c->sm_count * 16);
    k_face_keys<<<gr, TB, 0, st>>>(E, t, nb, c->dconn.p, hi.p, lo.p, slot.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    const int hi_bits = lv.w == 1 ? nb : 2 * nb;
    const int lo_bits = lv.w == 3 ? nb : 2 * nb;
    size_t tb_lo = 0, tb_hi = 0;
    if (lv.w >= 3) {
        ISL_CHECK_CUDA(c, ord1.alloc(n));
        ISL_CHECK_CUDA(c, hi2.alloc(n));
        cub::DeviceRadixSort::SortPairs(nullptr, tb_lo, lo.p, kout.p, slot.p, ord1.p, (int)n, 0, lo_bits, st);
    }
    cub::DeviceRadixSort::SortPairs(nullptr, tb_hi, hi.p, kout.p, slot.p, g.ord.p, (int)n, 0, hi_bits, st);
    DBuf<char> tmp;
    ISL_CHECK_CUDA(c, tmp.alloc(std::max<size_t>(std::max(tb_lo, tb_hi), 1)));
    if (lv.w >= 3) {
        // least significant part first; the radix sort is stable, so the second
        // pass keeps (lo, slot) order within equal hi
        size_t b = tb_lo;
        ISL_CHECK_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, b, lo.p, kout.p, slot.p, ord1.p, (int)n, 0, lo_bits, st));
        k_gather_key<<<gr, TB, 0, st>>>(n, ord1.p, hi.p, hi2.p);
        b = tb_hi;
        ISL_CHECK_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, b, hi2.p, kout.p, ord1.p, g.ord.p, (int)n, 0, hi_bits, st));
    } else {
        size_t b = tb_hi;
        ISL_CHECK_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, b, hi.p, kout.p, slot.p, g.ord.p, (int)n, 0, hi_bits, st));
    }
    // kout: hi keys in sorted order
    ISL_CHECK_CUDA(c, gs.alloc(n));
    ISL_CHECK_CUDA(c, g.head.alloc(n));
    k_heads<<<gr, TB, 0, st>>>(n, kout.p, lo.p, g.ord.p, gs.p, g.head.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 2 + (lv.w >= 3 ? 1 : 0);
    if (!need_first) {
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));  // the scratch buffers above are released on return
        return ISL_OK;
    }
    // group starts: inclusive max-scan of the head positions
    DBuf<int32_t> gstart;
    ISL_CHECK_CUDA(c, gstart.alloc(n));
    size_t sb = 0;
    cub::DeviceScan::InclusiveScan(nullptr, sb, gs.p, gstart.p, MaxOp(), (int)n, st);
    DBuf<char> stmp;
    ISL_CHECK_CUDA(c, stmp.alloc(std::max<size_t>(sb, 1)));
    ISL_CHECK_CUDA(c, cub::DeviceScan::InclusiveScan(stmp.p, sb, gs.p, gstart.p, MaxOp(), (int)n, st));
    ISL_CHECK_CUDA(c, g.first.alloc(n));
    ISL_CHECK_CUDA(c, g.flag.alloc(n + 1));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(g.flag.p + n, 0, sizeof(int32_t), st));
    k_first<<<gr, TB, 0, st>>>(n, g.ord.p, gstart.p, g.first.p, g.flag.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));  // the scratch buffers above are released on return
    c->launches += 1;
    return ISL_OK;
}

}  // namespace

bool device_setup_fits(const isl_ctx* c, int nfc) {
    return c->device >= 0 && c->nelem > 0 && (int64_t)c->nelem * nfc < (int64_t)INT32_MAX - 1 &&
           c->nnodes < ((int64_t)1 << 31);
}

int device_dofobj_numbering(isl_ctx* c, const std::vector<DeviceLevel>& levels, int nf) {
    cudaStream_t st = c->stream;
    const int64_t E = c->nelem;
    const int ninst = (int)c->ninst;
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));  // dedof of an earlier field may still be in use
    DBuf<int64_t> deoff, dbase;
    ISL_CHECK_CUDA(c, deoff.alloc(ninst + 1));
    ISL_CHECK_CUDA(c, dbase.alloc((size_t)ninst * std::max<size_t>(1, levels.size())));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(deoff.p, c->inst_elem_off.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    // per level: first occurrences and the exclusive scan of first visits
    std::vector<Groups> grp(levels.size());
    std::vector<DBuf<int32_t>> rank(levels.size());
    std::vector<std::vector<int64_t>> count(levels.size(), std::vector<int64_t>(ninst, 0));
    DBuf<int32_t> at;
    ISL_CHECK_CUDA(c, at.alloc(ninst + 1));
    std::vector<int32_t> hat(ninst + 1);
    for (size_t l = 0; l < levels.size(); ++l) {
        const DeviceLevel& lv = levels[l];
        if (lv.stride == 0) continue;
        if (lv.w == 0) {  // cell DOFs: one group per element
            for (int k = 0; k < ninst; ++k)
                count[l][k] = (c->inst_elem_off[k + 1] - c->inst_elem_off[k]) * lv.nfc;
            continue;
        }
        int rc = group_level(c, lv, grp[l], true);
        if (rc != ISL_OK) return rc;
        const int64_t n = E * lv.nfc;
        ISL_CHECK_CUDA(c, rank[l].alloc(n + 1));
        size_t sb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, sb, grp[l].flag.p, rank[l].p, (int)(n + 1), st);
        DBuf<char> stmp;
        ISL_CHECK_CUDA(c, stmp.alloc(std::max<size_t>(sb, 1)));
        ISL_CHECK_CUDA(c, cub::DeviceScan::ExclusiveSum(stmp.p, sb, grp[l].flag.p, rank[l].p, (int)(n + 1), st));
        k_rank_at<<<nblocks(ninst + 1), TB, 0, st>>>(ninst, deoff.p, lv.nfc, rank[l].p, at.p);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(hat.data(), at.p, (ninst + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
        c->launches += 1;
        for (int k = 0; k < ninst; ++k) count[l][k] = hat[k + 1] - hat[k];
    }
    // instance-major, then level order: the base id of every (level, instance)
    std::vector<int64_t> base((size_t)ninst * std::max<size_t>(1, levels.size()), 0);
    int64_t counter = 0;
    c->inst_dof_off.assign(ninst + 1, 0);
    for (int k = 0; k < ninst; ++k) {
        c->inst_dof_off[k] = counter;
        for (size_t l = 0; l < levels.size(); ++l) {
            base[l * ninst + k] = counter;
            counter += count[l][k] * levels[l].stride;
        }
    }
    c->inst_dof_off[ninst] = counter;
    if (counter >= INT32_MAX) ISL_FAIL(c, ISL_ERR_ARG, "too many DOF objects for 32-bit ids");
    c->ndofobj = counter;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(dbase.p, base.data(), base.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, c->dedof.alloc((size_t)E * nf));
    for (size_t l = 0; l < levels.size(); ++l) {
        const DeviceLevel& lv = levels[l];
        if (lv.stride == 0) continue;
        const int64_t n = E * lv.nfc;
        const unsigned gr = std::min<unsigned>(nblocks(n), (unsigned)c->sm_count * 16);
        if (lv.w == 0)
            k_assign_cell<<<gr, TB, 0, st>>>(E, lv.nfc * lv.stride, lv.begin, deoff.p, ninst, dbase.p + l * ninst, c->dedof.p);
        else
            k_assign<<<gr, TB, 0, st>>>(E, lv.nfc, lv.stride, lv.begin, grp[l].first.p, rank[l].p, deoff.p, ninst,
                                        dbase.p + l * ninst, c->dedof.p);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        c->launches += 1;
    }
    // host copy [E][nf] for the host-side steps (boundary points, constraints)
    DBuf<int32_t> aos;
    ISL_CHECK_CUDA(c, aos.alloc((size_t)E * nf));
    k_transpose<<<std::min<unsigned>(nblocks(E * nf), (unsigned)c->sm_count * 16), TB, 0, st>>>(E, nf, c->dedof.p, aos.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    std::vector<int32_t> h((size_t)E * nf);
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(h.data(), aos.p, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    c->launches += 1;
    c->hedof.resize(h.size());
    std::copy(h.begin(), h.end(), c->hedof.begin());
    return ISL_OK;
}

int device_boundary_slots(isl_ctx* c, const DeviceLevel& lv, std::vector<int64_t>& slots) {
    cudaStream_t st = c->stream;
    const int64_t n = c->nelem * lv.nfc;
    Groups g;
    int rc = group_level(c, lv, g, false);
    if (rc != ISL_OK) return rc;
    DBuf<uint8_t> single;
    DBuf<int32_t> sel, nsel;
    ISL_CHECK_CUDA(c, single.alloc(n));
    ISL_CHECK_CUDA(c, sel.alloc(n));
    ISL_CHECK_CUDA(c, nsel.alloc(1));
    k_single<<<std::min<unsigned>(nblocks(n), (unsigned)c->sm_count * 16), TB, 0, st>>>(n, g.head.p, single.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    size_t sb = 0;
    cub::DeviceSelect::Flagged(nullptr, sb, g.ord.p, single.p, sel.p, nsel.p, (int)n, st);
    DBuf<char> stmp;
    ISL_CHECK_CUDA(c, stmp.alloc(std::max<size_t>(sb, 1)));
    ISL_CHECK_CUDA(c, cub::DeviceSelect::Flagged(stmp.p, sb, g.ord.p, single.p, sel.p, nsel.p, (int)n, st));
    int32_t m = 0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&m, nsel.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    std::vector<int32_t> h((size_t)m);
    if (m > 0) {
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(h.data(), sel.p, (size_t)m * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    }
    c->launches += 2;
    slots.assign(h.begin(), h.end());
    return ISL_OK;
}

}  // namespace isl

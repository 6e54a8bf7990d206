// Cross-bucket link stage on sm_103a.
//
// Joins the partial unitigs of the merge (maximal within a sub-bucket) into maximal unitigs:
// the link semantics of GGCAT's extend_unitigs (crates/assembler_pipeline/src/extend_unitigs.rs:348-993),
// where a partial unitig end flagged as a sub-bucket boundary carries a "link" k-mer that is
// also the end of exactly one other partial unitig.
//
//   1. endpoints: the k-mer of every flagged end goes into a hash table, keyed like the build's
//      hash family (canonical, or as read for forward-only builds: the extremities are keyed
//      by hash.to_unextendable(), extend_unitigs.rs:142-147); per key the two smallest endpoint
//      ids (2*piece + side) are paired, the rest stay unpaired;
//   2. oriented nodes v = 2*piece + d (d = 0: stored orientation, entered by its left end;
//      d = 1: reverse complement): succ(v) = partner(v ^ 1), the endpoint entered next;
//   3. forward pointer jumping separates chains (every jump reaches an end) from cycles; the
//      cycle nodes get the smallest node of their cycle by min-label jumping, the copy whose
//      smallest node is even is cut before that node, the mirror copy is dropped;
//   4. predecessor pointer jumping gives every node its chain start and base offset; the end
//      node of the owning orientation (start <= mirror of its end) reserves the output;
//   5. one warp per node copies its bases (all of the start piece, the others without the k
//      bases they share with their predecessor), reverse-complemented for d = 1.
// A cut cycle drops its last base: its string then holds every k-mer once (circular flag).
#include "common.cuh"
#include "kernels.h"

namespace ggcat {

constexpr uint32_t kNoNode = 0xffffffffu;

__device__ __forceinline__ uint32_t ascii_code(uint8_t c) { return ((uint32_t)c >> 1) & 3u; }

template <typename KT>
__device__ __forceinline__ KT ascii_kmer(const uint8_t *s, int k) {
    KT v = 0;
    for (int i = 0; i < k; i++) v |= (KT)ascii_code(s[i]) << (2 * i);
    return v;
}

template <typename KT>
__global__ void __launch_bounds__(256) link_endpoints_kernel(const uint8_t *__restrict__ bases,
                                                             const uint64_t *__restrict__ off,
                                                             const uint32_t *__restrict__ len,
                                                             const uint8_t *__restrict__ flags, uint64_t n, int k,
                                                             int fwd, KT *keys, uint32_t *min1, uint64_t mask,
                                                             uint32_t *__restrict__ eslot, unsigned *status) {
    using K = KeyOps<KT>;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = e >> 1;
        const uint32_t side = (uint32_t)(e & 1);
        if (!(flags[i] & (1u << side))) {
            eslot[e] = kNoNode;
            continue;
        }
        const uint8_t *s = bases + off[i] + (side ? len[i] - (uint32_t)k : 0u);
        const KT fw = ascii_kmer<KT>(s, k);
        const KT rc = K::rc(fw, k);
        const KT key = (fwd || fw < rc) ? fw : rc;
        uint64_t slot = K::hash(key) & mask;
        uint32_t found = kNoNode;
        for (uint64_t probe = 0; probe <= mask; probe++) {
            bool created = false;
            const int r = slot_claim(&keys[slot], key, created);
            if (r > 0) {
                found = (uint32_t)slot;
                break;
            }
            if (r < 0) {
                atomicOr(status, kStatusWaitLimit);
                break;
            }
            slot = (slot + 1) & mask;
        }
        if (found == kNoNode) {
            atomicOr(status, kStatusTableFull);
            eslot[e] = kNoNode;
            continue;
        }
        atomicMin(&min1[found], (uint32_t)e);
        eslot[e] = found;
    }
}

__global__ void __launch_bounds__(256) link_second_kernel(const uint32_t *__restrict__ eslot,
                                                          const uint32_t *__restrict__ min1, uint32_t *min2,
                                                          uint64_t n_end) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_end;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = eslot[e];
        if (s != kNoNode && min1[s] != (uint32_t)e) atomicMin(&min2[s], (uint32_t)e);
    }
}

// succ(v) = partner of the endpoint v ^ 1 (the end v leaves by); J = succ or v itself
__global__ void __launch_bounds__(256) link_succ_kernel(const uint32_t *__restrict__ eslot,
                                                        const uint32_t *__restrict__ min1,
                                                        const uint32_t *__restrict__ min2, uint64_t nn,
                                                        uint32_t *__restrict__ succ, uint32_t *__restrict__ jump) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)v ^ 1u;
        const uint32_t s = eslot[x];
        uint32_t p = kNoNode;
        if (s != kNoNode) {
            const uint32_t a = min1[s], b = min2[s];
            if (b != kNoNode) p = x == a ? b : (x == b ? a : kNoNode);
        }
        succ[v] = p;
        jump[v] = p == kNoNode ? (uint32_t)v : p;
    }
}

// one forward jumping round; counts the nodes whose jump has not reached a chain end
__global__ void __launch_bounds__(256) link_jump_kernel(const uint32_t *__restrict__ succ,
                                                        const uint32_t *__restrict__ jump,
                                                        uint32_t *__restrict__ jump_n, uint64_t nn,
                                                        unsigned long long *unresolved) {
    unsigned long long cnt = 0;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = jump[v];
        const uint32_t jj = jump[j];
        jump_n[v] = jj;
        cnt += succ[jj] != kNoNode;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(unresolved, cnt);
}

// nodes still unresolved lie on cycles: compact them; cyc_jump starts as succ, cyc_min as
// min(v, succ(v))
__global__ void __launch_bounds__(256) link_cycle_list_kernel(const uint32_t *__restrict__ succ,
                                                              const uint32_t *__restrict__ jump, uint64_t nn,
                                                              uint32_t *__restrict__ list, unsigned long long *count,
                                                              uint32_t *__restrict__ cyc_jump,
                                                              uint32_t *__restrict__ cyc_min) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        if (succ[jump[v]] == kNoNode) continue;
        const unsigned long long i = atomicAdd(count, 1ull);
        list[i] = (uint32_t)v;
        cyc_jump[v] = succ[v];
        cyc_min[v] = min((uint32_t)v, succ[v]);
    }
}

// one min-label round over the cycle nodes (ping-pong arrays)
__global__ void __launch_bounds__(256) link_cycle_min_kernel(const uint32_t *__restrict__ list, uint64_t nc,
                                                             const uint32_t *__restrict__ cj,
                                                             const uint32_t *__restrict__ cm,
                                                             uint32_t *__restrict__ cj_n, uint32_t *__restrict__ cm_n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        const uint32_t j = cj[v];
        cm_n[v] = min(cm[v], cm[j]);
        cj_n[v] = cj[j];
    }
}

// cut: the copy of a cycle whose smallest node is even is cut before that node; the mirror
// copy (odd smallest node) is dropped
__global__ void __launch_bounds__(256) link_cycle_cut_kernel(const uint32_t *__restrict__ list, uint64_t nc,
                                                             const uint32_t *__restrict__ cm,
                                                             uint32_t *__restrict__ succ, uint8_t *__restrict__ node_state) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = list[i];
        const uint32_t mn = cm[v];
        if (mn & 1u) {
            node_state[v] = 2;  // dropped
        } else {
            node_state[v] = 1;  // on a cut cycle
            if (succ[v] == mn) succ[v] = kNoNode;
        }
    }
}

// predecessor jumping start: pjump = v, prank = 0 (no predecessor) ...
__global__ void __launch_bounds__(256) link_pred_reset_kernel(uint64_t nn, uint32_t *__restrict__ pjump,
                                                              unsigned long long *__restrict__ prank) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        pjump[v] = (uint32_t)v;
        prank[v] = 0;
    }
}

// ... then pjump = pred, prank = the bases the predecessor contributes
__global__ void __launch_bounds__(256) link_pred_init_kernel(const uint32_t *__restrict__ succ,
                                                             const uint8_t *__restrict__ node_state,
                                                             const uint32_t *__restrict__ len, uint64_t nn, int k,
                                                             uint32_t *__restrict__ pjump,
                                                             unsigned long long *__restrict__ prank) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = succ[v];
        if (s == kNoNode || node_state[v] == 2) continue;
        pjump[s] = (uint32_t)v;
        prank[s] = (unsigned long long)(len[v >> 1] - (uint32_t)k);
    }
}

__global__ void __launch_bounds__(256) link_pred_jump_kernel(const uint32_t *__restrict__ pj,
                                                             const unsigned long long *__restrict__ pr,
                                                             uint32_t *__restrict__ pj_n,
                                                             unsigned long long *__restrict__ pr_n, uint64_t nn,
                                                             unsigned long long *changed) {
    unsigned long long cnt = 0;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = pj[v];
        const uint32_t jj = pj[j];
        pr_n[v] = pr[v] + pr[j];
        pj_n[v] = jj;
        cnt += jj != j;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(changed, cnt);
}

// The end node of every owned chain reserves its output: chain_off[start] = base offset.
__global__ void __launch_bounds__(256) link_reserve_kernel(
    const uint32_t *__restrict__ succ, const uint8_t *__restrict__ node_state, const uint32_t *__restrict__ pj,
    const unsigned long long *__restrict__ pr, const uint32_t *__restrict__ len, const uint8_t *__restrict__ pflags,
    uint64_t nn, unsigned long long *__restrict__ chain_off, uint64_t *__restrict__ u_off, uint32_t *__restrict__ u_len,
    uint8_t *__restrict__ u_flags, unsigned long long *counters, unsigned long long bases_cap,
    unsigned long long u_cap, unsigned *status) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nn;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t st = node_state[v];
        if (st == 2 || succ[v] != kNoNode) continue;  // not an end node
        const uint32_t start = pj[v];
        bool owner;
        if (st == 1)
            owner = true;  // the kept copy of a cut cycle
        else
            owner = start <= ((uint32_t)v ^ 1u);  // a chain and its mirror: the one starting lower
        if (!owner) continue;
        const unsigned long long total = pr[v] + len[v >> 1];
        const unsigned long long off = atomicAdd(&counters[0], total);
        const unsigned long long idx = atomicAdd(&counters[1], 1ull);
        if (off + total > bases_cap || idx >= u_cap) {
            atomicOr(status, kStatusOutOverflow);
            continue;
        }
        chain_off[start] = off;
        u_off[idx] = off;
        u_len[idx] = (uint32_t)(st == 1 ? total - 1 : total);
        uint8_t f = 0;
        if (st == 1)
            f = 4;
        else if (start == ((uint32_t)v & ~1u) && start == (uint32_t)v && !(pflags[v >> 1] & 3u))
            f = pflags[v >> 1] & 4u;  // an unlinked piece keeps its in-sub-bucket circular flag
        u_flags[idx] = f;
    }
}

__device__ __forceinline__ uint8_t comp_ascii(uint8_t c) {
    return c == 'A' ? 'T' : c == 'T' ? 'A' : c == 'C' ? 'G' : 'C';
}

// one warp per node: copy its bases into its chain's output
__global__ void __launch_bounds__(256) link_write_kernel(const uint8_t *__restrict__ bases,
                                                         const uint64_t *__restrict__ off,
                                                         const uint32_t *__restrict__ len,
                                                         const uint8_t *__restrict__ node_state,
                                                         const uint32_t *__restrict__ pj,
                                                         const unsigned long long *__restrict__ pr,
                                                         const unsigned long long *__restrict__ chain_off, uint64_t nn,
                                                         int k, uint8_t *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t v = warp; v < nn; v += n_warps) {
        if (node_state[v] == 2) continue;
        const uint32_t start = pj[v];
        const unsigned long long base = chain_off[start];
        if (base == ~0ull) continue;  // the mirror copy of an owned chain
        const uint64_t i = v >> 1;
        const uint32_t L = len[i];
        const bool first = start == (uint32_t)v;
        const uint32_t from = first ? 0u : (uint32_t)k;
        const unsigned long long dst = base + (first ? 0ull : pr[v] + (unsigned long long)k);
        const uint8_t *src = bases + off[i];
        if ((v & 1) == 0) {
            for (uint32_t j = from + (uint32_t)lane; j < L; j += 32) out[dst + j - from] = src[j];
        } else {
            for (uint32_t j = from + (uint32_t)lane; j < L; j += 32) out[dst + j - from] = comp_ascii(src[L - 1 - j]);
        }
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static unsigned grid_for(uint64_t n, int sms) {
    const uint64_t b = (n + 255) / 256;
    const uint64_t cap = (uint64_t)sms * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, cap));
}

int launch_link_endpoints(const uint8_t *bases, const uint64_t *off, const uint32_t *len, const uint8_t *flags,
                          uint64_t n, int k, int fwd, void *keys, uint32_t *min1, uint64_t mask, uint32_t *eslot,
                          unsigned *status, int sms, cudaStream_t s) {
    if (n == 0) return 0;
    if (k > 64)
        link_endpoints_kernel<u256><<<grid_for(2 * n, sms), 256, 0, s>>>(
            bases, off, len, flags, n, k, fwd, static_cast<u256 *>(keys), min1, mask, eslot, status);
    else if (k > 32)
        link_endpoints_kernel<u128><<<grid_for(2 * n, sms), 256, 0, s>>>(
            bases, off, len, flags, n, k, fwd, static_cast<u128 *>(keys), min1, mask, eslot, status);
    else
        link_endpoints_kernel<uint64_t><<<grid_for(2 * n, sms), 256, 0, s>>>(
            bases, off, len, flags, n, k, fwd, static_cast<uint64_t *>(keys), min1, mask, eslot, status);
    link_second_kernel<<<grid_for(2 * n, sms), 256, 0, s>>>(eslot, min1, min1 + (mask + 1), 2 * n);
    return 2;
}

int launch_link_succ(const uint32_t *eslot, const uint32_t *min1, const uint32_t *min2, uint64_t nn,
                     uint32_t *succ, uint32_t *jump, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_succ_kernel<<<grid_for(nn, sms), 256, 0, s>>>(eslot, min1, min2, nn, succ, jump);
    return 1;
}

int launch_link_jump(const uint32_t *succ, const uint32_t *jump, uint32_t *jump_n, uint64_t nn,
                     unsigned long long *unresolved, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_jump_kernel<<<grid_for(nn, sms), 256, 0, s>>>(succ, jump, jump_n, nn, unresolved);
    return 1;
}

int launch_link_cycle_list(const uint32_t *succ, const uint32_t *jump, uint64_t nn, uint32_t *list,
                           unsigned long long *count, uint32_t *cyc_jump, uint32_t *cyc_min, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_cycle_list_kernel<<<grid_for(nn, sms), 256, 0, s>>>(succ, jump, nn, list, count, cyc_jump, cyc_min);
    return 1;
}

int launch_link_cycle_min(const uint32_t *list, uint64_t nc, const uint32_t *cj, const uint32_t *cm, uint32_t *cj_n,
                          uint32_t *cm_n, int sms, cudaStream_t s) {
    if (nc == 0) return 0;
    link_cycle_min_kernel<<<grid_for(nc, sms), 256, 0, s>>>(list, nc, cj, cm, cj_n, cm_n);
    return 1;
}

int launch_link_cycle_cut(const uint32_t *list, uint64_t nc, const uint32_t *cm, uint32_t *succ, uint8_t *node_state,
                          int sms, cudaStream_t s) {
    if (nc == 0) return 0;
    link_cycle_cut_kernel<<<grid_for(nc, sms), 256, 0, s>>>(list, nc, cm, succ, node_state);
    return 1;
}

int launch_link_pred_init(const uint32_t *succ, const uint8_t *node_state, const uint32_t *len, uint64_t nn, int k,
                          uint32_t *pjump, unsigned long long *prank, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_pred_reset_kernel<<<grid_for(nn, sms), 256, 0, s>>>(nn, pjump, prank);
    link_pred_init_kernel<<<grid_for(nn, sms), 256, 0, s>>>(succ, node_state, len, nn, k, pjump, prank);
    return 2;
}

int launch_link_pred_jump(const uint32_t *pj, const unsigned long long *pr, uint32_t *pj_n, unsigned long long *pr_n,
                          uint64_t nn, unsigned long long *changed, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_pred_jump_kernel<<<grid_for(nn, sms), 256, 0, s>>>(pj, pr, pj_n, pr_n, nn, changed);
    return 1;
}

int launch_link_reserve(const uint32_t *succ, const uint8_t *node_state, const uint32_t *pj,
                        const unsigned long long *pr, const uint32_t *len, const uint8_t *pflags, uint64_t nn,
                        unsigned long long *chain_off, uint64_t *u_off, uint32_t *u_len, uint8_t *u_flags,
                        unsigned long long *counters, unsigned long long bases_cap, unsigned long long u_cap,
                        unsigned *status, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_reserve_kernel<<<grid_for(nn, sms), 256, 0, s>>>(succ, node_state, pj, pr, len, pflags, nn, chain_off, u_off,
                                                          u_len, u_flags, counters, bases_cap, u_cap, status);
    return 1;
}

int launch_link_write(const uint8_t *bases, const uint64_t *off, const uint32_t *len, const uint8_t *node_state,
                      const uint32_t *pj, const unsigned long long *pr, const unsigned long long *chain_off,
                      uint64_t nn, int k, uint8_t *out, int sms, cudaStream_t s) {
    if (nn == 0) return 0;
    link_write_kernel<<<(unsigned)((uint64_t)sms * 16), 256, 0, s>>>(bases, off, len, node_state, pj, pr, chain_off,
                                                                     nn, k, out);
    return 1;
}

}  // namespace ggcat

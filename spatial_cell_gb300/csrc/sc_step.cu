// sc_step.cu -- the step's kernels on sm_103a, one per reference kernel.
//
// Each kernel computes, for every item it owns, exactly the floating-point
// expression sequence of the reference kernel named in its comment (same
// operand order, same implicit double-precision literals, no fused
// multiply-add: the file is built with -fmad=false), so its results are
// bit-identical to the reference's on the same input state.  What changes is
// where the data lives: structure-of-arrays fields read 16 bytes at a time,
// double buffering only for the fields a kernel's neighbours read, elementwise
// kernels updating in place, and no memset of a whole 256-byte-per-item
// buffer before each kernel (main.cu:326-638 does 92 of them per step).
//
// Launch shape: one thread per slot, 256 threads per CTA; the bound of every
// kernel is the device-side active counter, so no host round trip is needed
// between kernels (the reference reads nActiveParticles back three times per
// step, main.cu:369,399,616).
#include "sc_launch.h"
#include "sc_tile.cuh"

__device__ __forceinline__ bool p_order(int ta, int ia, int tb, int ib) { return ta < tb || (ta == tb && ia < ib); }

// ---- dynamics.cuh:19-215: move (its only live effect: debugVector.xyz = 0)
// fused with brownianMovementAndRotation, in place --------------------------------
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_move_brownian(const int *__restrict__ nActivePtr,
                                                              const int4 *__restrict__ info,
                                                              const float4 *__restrict__ pos, float4 *dbg,
                                                              float4 *posnoise, float4 *angnoise, ScParams P,
                                                              float scale, uint32_t su, uint32_t sn,
                                                              const int *__restrict__ stepPtr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    const int step = *stepPtr;
    int4 in = info[i];
    if (!(in.z & SC_ACTIVE)) return;
    rep_apply<BATCH>(P, in.w);
    float4 d = dbg[i];
    d.x = 0.0f; d.y = 0.0f; d.z = 0.0f;
    dbg[i] = d;
    float radius = pos[i].w;
    uint32_t id = (uint32_t)in.x, st = (uint32_t)step;
    uint64_t seed = P.seed;
    sc_f4 r1 = sc_random_rotation(sc_uniform(seed, su, id, st, 0), sc_uniform(seed, su, id, st, 1),
                                  sc_uniform(seed, su, id, st, 2));
    float nrm = sc_normal(seed, sn, id, st, 0);
    float mag = sc_noise_mag(fabsf(nrm) * scale, radius);
    st3(posnoise, i, sc_rotate(sc_up(), r1) * mag, 0.0f);
    sc_f4 r2 = sc_random_rotation(sc_uniform(seed, su, id, st, 3), sc_uniform(seed, su, id, st, 4),
                                  sc_uniform(seed, su, id, st, 5));
    float t = sc_rot_noise(P.rotNoise, radius);
    st4(angnoise, i, sc_slerp(ld4(angnoise, i), r2, t));
}

// ---- dynamics.cuh:217-242 applyNoise, in place -------------------------------
__global__ void __launch_bounds__(SC_THREADS) k_apply_noise(const int *__restrict__ nActivePtr,
                                                            const int4 *__restrict__ info, float4 *vel,
                                                            float4 *posnoise, float4 *angvel, float4 *angnoise) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    if (!(info[i].z & SC_ACTIVE)) return;
    sc_f3 v = ld3(vel, i);
    v += ld3(posnoise, i);
    st3(vel, i, v, 0.0f);
    st3(posnoise, i, sc_zero3(), 0.0f);
    st4(angvel, i, sc_qmul(ld4(angnoise, i), ld4(angvel, i)));
    st4(angnoise, i, sc_qid());
}

// ---- dynamics.cuh:244-282 applyVelocities, in place ---------------------------
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_apply_velocities(const int *__restrict__ nActivePtr,
                                                                 const int4 *__restrict__ info, float4 *pos,
                                                                 float4 *vel, float4 *rot, float4 *angvel,
                                                                 ScParams P, float f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    const int4 in = info[i];
    if (!(in.z & SC_ACTIVE)) return;
    rep_apply<BATCH>(P, in.w);
    float4 p4 = pos[i];
    sc_f3 p = sc_make_f3(p4.x, p4.y, p4.z);
    sc_f3 v = ld3(vel, i);
    p = P.periodic ? sc_wrap3(p + v * f, P.simSize)
                   : (P.walls ? sc_reflect3(p + v * f, P.simSize) : clamp(p + v * f, 0.0f, P.simSize));
    v *= P.velDecay;
    sc_f4 av = ld4(angvel, i);
    sc_f4 r = sc_qmul(sc_slerp(sc_qid(), av, f), ld4(rot, i));
    r /= length(r);
    av = sc_slerp(av, sc_qid(), 1.0f - P.angDecay);
    pos[i] = make_float4(p.x, p.y, p.z, p4.w);
    st3(vel, i, v, 0.0f);
    st4(rot, i, r);
    st4(angvel, i, av);
}

// ---- pair lists ------------------------------------------------------------------
// The list of item i is read as entries list[k * cap + i], k < cnt[i]; cnt[i]
// above the list's capacity means "scan instead".
template <int K>
struct PairList {
    const uint32_t *__restrict__ list;
    const int *__restrict__ cnt;
    int cap;
    const int *__restrict__ perm;  // position -> item (count-ordered lists; null: identity)
};

// Packed 32-bit list entries: 4 consecutive entries of an item share one
// 16-byte chunk, chunks warp-tiled (chunk q of position g at
// ((g/32) * K/4 + q) * 32 + g%32), so one load brings 4 entries.
__host__ __device__ __forceinline__ size_t sc_list4_at(int K, int g, int k) {
    return (((size_t)(g >> 5) * (size_t)(K / 4) + (size_t)(k >> 2)) * 32 + (size_t)(g & 31)) * 4 + (size_t)(k & 3);
}
__device__ __forceinline__ const uint4 *sc_list4_chunks(const uint32_t *list, int K, int g) {
    return reinterpret_cast<const uint4 *>(list) + (size_t)(g >> 5) * (size_t)(K / 4) * 32 + (size_t)(g & 31);
}

// Count-ordered list layout.  A builder block first writes each item's list
// at the item's own position of `scratch`; this re-orders the block's items
// by descending list length and copies the lists to their new positions, so
// a consumer warp walks lists of similar lengths; the lists are written
// packed (sc_list4_at).  perm[g] is the item at
// position g (-1 past the last item), cnt[g] its list length.  Every thread
// of the block must call it.  `scratch` is written earlier in the same kernel
// by other threads of the block, so it is read through a plain (coherent)
// pointer after the barrier.
// The block's ranking by descending list length: thread t takes position
// b0 + t, whose item is b0 + *src (list length *cs, -1 past the last item).
template <int K>
__device__ __forceinline__ void count_rank(bool valid, int c, int *src, int *cs) {
    __shared__ int hist[K + 3];
    __shared__ int s_cnt[SC_THREADS], s_src[SC_THREADS];
    const int t = threadIdx.x;
    for (int b = t; b < K + 3; b += SC_THREADS) hist[b] = 0;
    s_cnt[t] = valid ? c : -1;
    __syncthreads();
    const int bin = valid ? 1 + min(c, K + 1) : 0;
    const int idx = atomicAdd(&hist[bin], 1);
    __syncthreads();
    if (t < 32) {  // exclusive prefix over bins, highest bin first
        int carry = 0;
        for (int top = K + 2; top >= 0; top -= 32) {
            const int b = top - t;
            const int v = b >= 0 ? hist[b] : 0;
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, x, o);
                if (t >= o) x += y;
            }
            if (b >= 0) hist[b] = carry + x - v;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
    }
    __syncthreads();
    s_src[hist[bin] + idx] = t;
    __syncthreads();
    *src = s_src[t];
    *cs = s_cnt[*src];
}

template <int K>
__device__ __forceinline__ void emit_count_ordered(bool valid, int c, int limit, int cap,
                                                   const uint32_t *scratch, uint32_t *__restrict__ list,
                                                   int *__restrict__ cnt, int *__restrict__ perm,
                                                   int *__restrict__ ovf = nullptr, int *__restrict__ ovfCount = nullptr) {
    const int b0 = blockIdx.x * SC_THREADS;
    int src, cs;
    count_rank<K>(valid, c, &src, &cs);
    const int g = b0 + threadIdx.x;
    if (g < cap) {
        perm[g] = cs >= 0 ? b0 + src : -1;
        cnt[g] = max(cs, 0);
    }
    const int n = min(max(cs, 0), min(K, limit));
    for (int k = 0; k < n; k++) list[sc_list4_at(K, g, k)] = scratch[sc_list_at(K, b0 + src, k)];
    if (ovf && cs > min(K, limit)) ovf[atomicAdd(ovfCount, 1)] = g;
}

// Bonds of one particle held in registers, with a one-word filter of the
// partner ids (bit id mod 32 set for each bond) that rules most candidates
// out before the slot-by-slot comparison.
struct BondRegs {
    int n;
    uint32_t filter;
    int t[SC_MAX_ACTIVE_INTERACTIONS], g[SC_MAX_ACTIVE_INTERACTIONS], p[SC_MAX_ACTIVE_INTERACTIONS];
    __device__ __forceinline__ void load(const int *__restrict__ nb, const int *__restrict__ bonds, int i) {
        n = min(max(nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
        filter = 0u;
#pragma unroll
        for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++) {
            const int *b = bonds + (size_t)i * 24 + 3 * k;
            t[k] = k < n ? b[0] : 0;
            g[k] = k < n ? b[1] : 0;
            p[k] = k < n ? b[2] : 0;
            if (k < n) filter |= 1u << (p[k] & 31);
        }
    }
    __device__ __forceinline__ bool has_partner(int id) const {
        if (!((filter >> (id & 31)) & 1u)) return false;
        bool r = false;
#pragma unroll
        for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++)
            if (k < n && p[k] == id) r = true;
        return r;
    }
};

// The tests of a candidate inside the interaction cube: returns the entry
// flags, 0 if the pair contributes nothing.
__device__ __forceinline__ uint32_t pp_flags_in_cube(sc_f3 delta, float trad, int j, float prad, int phydro,
                                                     const BondRegs &B, const int4 *__restrict__ info) {
    int4 tin = info[j];
    if (!(tin.z & SC_ACTIVE)) return 0;
    float dist = sc_norm3(delta);
    float s = prad + trad;
    int thydro = (int)(int8_t)(tin.w & 0xff);
    uint32_t f = 0;
    if ((phydro > 0 || thydro > 0) && sc_within_lipid_range(dist, s) && phydro == SC_POLAR && thydro == SC_POLAR)
        f |= SC_PP_POLAR;
    bool partner = B.has_partner(tin.x);
    if (partner) f |= SC_PP_PARTNER;
    if (!partner && dist < s) f |= SC_PP_COLLIDE;
    return f;
}

// The position-only tests of relax for candidate j of particle i
// (dynamics.cuh:452-478, 584-589, 775-777): returns the entry flags, 0 if
// the pair contributes nothing.
__device__ __forceinline__ uint32_t pp_flags(const ScParams &P, const Imager &IM, int i, int j, sc_f3 ppos, float prad,
                                             int phydro,
                                             const BondRegs &B, const float4 *__restrict__ pos,
                                             const int4 *__restrict__ info) {
    if (j == i) return 0;
    // the cube test first: most candidates fail it, and then need no record
    float4 t4 = pos[j];
    sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - ppos;
    if (outside_cube(delta, P.maxInt)) return 0;
    return pp_flags_in_cube(delta, t4.w, j, prad, phydro, B, info);
}

// Particle-particle list, built once after the sort; read by coordinateNoise
// and relax.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_pp(ScParams P, const uint32_t *__restrict__ cellStart,
                                                         const int *__restrict__ nActivePtr,
                                                         const float4 *__restrict__ pos, const int4 *__restrict__ info,
                                                         const int *__restrict__ nb, const int *__restrict__ bonds,
                                                         uint32_t *__restrict__ list, int *__restrict__ cnt, int cap,
                                                         int *__restrict__ classIdx, int *__restrict__ classCount,
                                                         int *__restrict__ ovf, int *__restrict__ ovfCount,
                                                         uint32_t *__restrict__ match, int *__restrict__ matchN) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    int4 in = info[i];
    int cls = 2;
    if (!(in.z & SC_ACTIVE)) {
        cnt[i] = 0;
    } else {
        rep_apply<BATCH>(P, in.w);
        BondRegs B;
        B.load(nb, bonds, i);
        float4 p4 = pos[i];
        const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, ppos, SC_BINNED_P);
        const int phydro = (int)(int8_t)(in.w & 0xff);
        int c = 0, nm = 0;
        uint32_t any = 0;
        uint32_t *__restrict__ myMatch = match + (size_t)i * SC_MAX_ACTIVE_INTERACTIONS;
        const int K = min(SC_LIST_PP, P.listLimit);
        auto add = [&](int j, uint32_t f) {
            if (c < K) list[sc_list_at(SC_LIST_PP, i, c)] = (uint32_t)j | f;
            c++;
            any |= f;
            if (f & SC_PP_PARTNER) {  // the bond slots naming this neighbour, in slot order
                const int tid_ = info[j].x;
#pragma unroll
                for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++)
                    if (k < B.n && B.p[k] == tid_ && nm < SC_MAX_ACTIVE_INTERACTIONS)
                        myMatch[nm++] = (uint32_t)j | ((uint32_t)k << 29);
            }
        };
        // 1. the candidates inside the interaction cube, in visiting order, held in the list's
        // slots (a cheap loop: most candidates leave at the cube test)
        int pc = 0;
        scan27(P, cellStart, ppos, reach(P, ppos, P.maxInt, SC_BINNED_P), [&](int j) {
            if (j == i) return;
            const float4 t4 = pos[j];
            if (outside_cube(IM(sc_make_f3(t4.x, t4.y, t4.z)) - ppos, P.maxInt)) return;
            if (pc < K) list[sc_list_at(SC_LIST_PP, i, pc)] = (uint32_t)j;
            pc++;
        });
        if (pc <= K) {
            // 2. their remaining tests in order, the list compacted in place (entry c <= k)
            for (int k = 0; k < pc; k++) {
                const int j = (int)list[sc_list_at(SC_LIST_PP, i, k)];
                const float4 t4 = pos[j];
                const sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - ppos;
                const uint32_t f = pp_flags_in_cube(delta, t4.w, j, p4.w, phydro, B, info);
                if (f) add(j, f);
            }
        } else {
            // more in-cube candidates than the list holds: every test in one scan
            scan27(P, cellStart, ppos, reach(P, ppos, P.maxInt, SC_BINNED_P), [&](int j) {
                const uint32_t f = pp_flags(P, IM, i, j, ppos, p4.w, phydro, B, pos, info);
                if (f) add(j, f);
            });
        }
        cnt[i] = c;
        // A test bond rotates the particle itself, which its later terms
        // read: its relaxation takes the in-order scan with the overflowed
        // items (its noise stays with the bonded class).
        bool testBond = false;
#pragma unroll
        for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++) testBond |= k < B.n && B.t[k] == 0;
        if (B.n >= 1) matchN[i] = nm | (testBond ? SC_MATCH_INORDER : 0);
        if (c > min(SC_LIST_PP, P.listLimit) || testBond) ovf[atomicAdd(ovfCount, 1)] = i;
        if (B.n >= 1) cls = 0;
        else if (c <= min(SC_LIST_PP, P.listLimit) && (any & SC_PP_POLAR)) cls = 1;
    }
    // append i to its class (warp-aggregated; order within a class is free)
    unsigned same = __match_any_sync(__activemask(), cls);
    int leader = __ffs(same) - 1, lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(&classCount[cls], __popc(same));
    base = __shfl_sync(same, base, leader);
    classIdx[(size_t)cls * cap + base + __popc(same & ((1u << lane) - 1u))] = i;
}

// Visits the contributing pairs of particle i in the reference's order: from
// the list, or (list overflow) by scanning.
template <class F>
__device__ __forceinline__ void for_pp(const ScParams &P, const uint32_t *__restrict__ cellStart,
                                       const PairList<SC_LIST_PP> &L, int i, sc_f3 ppos, float prad, int phydro,
                                       const int *__restrict__ nb, const int *__restrict__ bonds,
                                       const float4 *__restrict__ pos, const int4 *__restrict__ info, F &&f) {
    int c = L.cnt[i];
    if (c <= min(SC_LIST_PP, P.listLimit)) {
        for (int k = 0; k < c; k++) {
            uint32_t e = L.list[sc_list_at(SC_LIST_PP, i, k)];
            f((int)(e & SC_PP_INDEX), e);
        }
    } else {
        const Imager IM(P, ppos, SC_BINNED_P);
        BondRegs B;
        B.load(nb, bonds, i);
        scan27(P, cellStart, ppos, reach(P, ppos, P.maxInt, SC_BINNED_P), [&](int j) {
            uint32_t fl = pp_flags(P, IM, i, j, ppos, prad, phydro, B, pos, info);
            if (fl) f(j, fl);
        });
    }
}

// ---- dynamics.cuh:288-402 coordinateNoise -----------------------------------
// Only interaction partners change anything: for a listed item they are its
// bond matches (k_build_pp), in the reference's visiting order; an item
// whose list overflowed scans its neighbourhood.
// dynamics.cuh:288-402 for one particle; the new noise goes to pnOut / anOut.
template <bool BATCH>
__device__ __forceinline__ void coordinate_noise_item(
    const ScParams &P0, const uint32_t *__restrict__ cellStart, int i, const float4 *__restrict__ pos,
    const int4 *__restrict__ info, const int *__restrict__ nb, const int *__restrict__ bonds,
    const PairList<SC_LIST_PP> &L, const uint32_t *__restrict__ match, const int *__restrict__ matchN,
    const float4 *__restrict__ pnIn, const float4 *__restrict__ anIn, float4 *__restrict__ pnOut,
    float4 *__restrict__ anOut, float frac) {
    int4 in = info[i];
    float4 pn4 = pnIn[i], an4 = anIn[i];
    if (!(in.z & SC_ACTIVE) || nb[i] < 1) {
        *pnOut = pn4;
        *anOut = an4;
        return;
    }
    ScParams P = P0;
    rep_apply<BATCH>(P, in.w);
    const int nbi = min(max(nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
    const int *__restrict__ myBonds = bonds + (size_t)i * 24;
    float4 p4 = pos[i];
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const float prad = p4.w;
    sc_f3 ppn = sc_make_f3(pn4.x, pn4.y, pn4.z);
    sc_f4 pan = sc_make_f4(an4.x, an4.y, an4.z, an4.w);
    sc_f3 dPN = sc_zero3();
    sc_f4 dAN = sc_qid();
    float w = 0.0f;
    // one bond slot k naming neighbour j
    auto term = [&](int j, int k) {
        if (myBonds[3 * k] < 10 && frac > 0.25f) return;
        const float trad = pos[j].w;
        sc_f3 tpn = ld3(pnIn, j);
        sc_f4 tan_ = ld4(anIn, j);
        float pMag = length(ppn);
        dPN += (tpn - ppn) * 0.9f * trad / (prad + trad) * 1.0f;
        dPN *= fmaxf(length(dPN), pMag) / length(dPN);
        dAN = sc_slerp(dAN, sc_qmul(sc_qinv(pan), tan_), 0.9f * trad / (prad + trad) * 1.0f);
        w += 1.0f;
    };
    if (L.cnt[i] <= min(SC_LIST_PP, P.listLimit)) {
        const uint32_t *__restrict__ myMatch = match + (size_t)i * SC_MAX_ACTIVE_INTERACTIONS;
        const int nm = matchN[i] & SC_MATCH_COUNT;
        for (int m = 0; m < nm; m++) {
            const uint32_t e = myMatch[m];
            term((int)(e & SC_PP_INDEX), (int)(e >> 29));
        }
    } else {
        for_pp(P, cellStart, L, i, ppos, prad, (int)(int8_t)(in.w & 0xff), nb, bonds, pos, info,
               [&](int j, uint32_t fl) {
                   if (!(fl & SC_PP_PARTNER)) return;
                   const int tid_ = info[j].x;
#pragma unroll 1
                   for (int k = 0; k < nbi; k++)
                       if (myBonds[3 * k + 2] == tid_) term(j, k);
               });
    }
    ppn += dPN / fmaxf(w, 1.0f);
    pan = sc_qmul(sc_slerp(sc_qid(), dAN, 1.0f / fmaxf(w, 1.0f)), pan);
    st3(pnOut, 0, ppn, pn4.w);
    st4(anOut, 0, pan);
}


// Runs over the bonded work class (items with at least one bond), the new
// noise of class position t going to pnTmp[t] / anTmp[t]; every other
// item's noise is unchanged.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_coordinate_noise(
    ScParams P, const uint32_t *__restrict__ cellStart, const int *__restrict__ classIdx,
    const int *__restrict__ classCount, const float4 *__restrict__ pos, const int4 *__restrict__ info,
    const int *__restrict__ nb, const int *__restrict__ bonds, PairList<SC_LIST_PP> L,
    const uint32_t *__restrict__ match, const int *__restrict__ matchN, const float4 *__restrict__ pnIn,
    const float4 *__restrict__ anIn, float4 *__restrict__ pnTmp, float4 *__restrict__ anTmp, float frac) {
    const int n0 = classCount[0];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n0; t += gridDim.x * blockDim.x)
        coordinate_noise_item<BATCH>(P, cellStart, classIdx[t], pos, info, nb, bonds, L, match, matchN, pnIn, anIn,
                              pnTmp + t, anTmp + t, frac);
}

// The bonded class's new noise written back in place (after every read of
// the old values).
__global__ void __launch_bounds__(SC_THREADS) k_noise_writeback(const int *__restrict__ classIdx,
                                                                const int *__restrict__ classCount,
                                                                const float4 *__restrict__ pnTmp,
                                                                const float4 *__restrict__ anTmp,
                                                                float4 *__restrict__ pn, float4 *__restrict__ an) {
    const int n0 = classCount[0];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n0; t += gridDim.x * blockDim.x) {
        const int i = classIdx[t];
        pn[i] = pnTmp[t];
        an[i] = anTmp[t];
    }
}

// ---- dynamics.cuh:405-822 relax ------------------------------------------------
struct RelaxArgs {
    const uint32_t *__restrict__ cellStart;
    const int *__restrict__ nActivePtr;
    const float4 *__restrict__ pos;
    const int4 *__restrict__ info;
    const int *__restrict__ nb;
    const int *__restrict__ bonds;
    PairList<SC_LIST_PP> L;
    const float4 *__restrict__ velIn, *__restrict__ rotIn, *__restrict__ avIn;
    float4 *__restrict__ velOut, *__restrict__ rotOut, *__restrict__ avOut, *__restrict__ dbg;
    const int *__restrict__ classIdx;    // items by work class (k_build_pp)
    const int *__restrict__ classCount;
    const uint32_t *__restrict__ match;  // bond matches of the list (k_build_pp)
    const int *__restrict__ matchN;
};

// One particle's relaxation.  SCAN = false reads the particle's pair list;
// SCAN = true (list overflow) visits its 27 cells and applies the list's
// tests to each candidate.  MODE is the particle's work class: 0 all pair
// kinds, 1 no bond partners, 2 collisions only (the class guarantees the
// list holds no other kinds).  The bond loop reads the particle's bonds from
// memory one at a time, so its body is emitted once.
#define SC_PLAIN_GROUP 4
template <bool SCAN, int MODE>
__device__ __forceinline__ void relax_item(const ScParams &P, const RelaxArgs &A, int i, int4 in, float4 v4, float4 r4,
                                           float4 a4) {
    float4 p4 = A.pos[i];
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, ppos, SC_BINNED_P);
    const float prad = p4.w;
    const sc_f3 pvel = sc_make_f3(v4.x, v4.y, v4.z);
    sc_f4 prot = sc_make_f4(r4.x, r4.y, r4.z, r4.w);
    sc_f4 pav = sc_make_f4(a4.x, a4.y, a4.z, a4.w);
    const int pid = in.x, ptype = in.y, phydro = (int)(int8_t)(in.w & 0xff);
    const int nbi = min(max(A.nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
    const int *__restrict__ myBonds = A.bonds + (size_t)i * 24;
    sc_f4 pdbg = sc_make_f4(0, 0, 0, 0);
    bool dbgTouched = false;
    sc_f3 dV = sc_zero3();
    sc_f4 dAV = sc_qid();
    sc_f3 phobPos = sc_zero3();
    float phobSum = 0.0f;
    float w = 0.0f;
    const sc_f3 up = sc_rotate(sc_up(), prot);
    const sc_f3 nextUp = sc_rotate(up, pav);
    const float flex = SC_PI_REF / 8;
    auto body = [&](int j, uint32_t fl) {
        float4 t4 = A.pos[j];
        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
        const float trad = t4.w;
        const float idist = prad + trad;
        if (MODE <= 1 && (fl & SC_PP_POLAR)) {
            // dynamics.cuh:478-582: polar (lipid) head / tail attraction
            sc_f3 tvel = ld3(A.velIn, j);
            sc_f3 nextTup = sc_rotate(sc_rotate(sc_up(), ld4(A.rotIn, j)), pav);
            sc_f3 pPV = -nextUp * prad + ppos + pvel;
            sc_f3 tpPV = -nextTup * trad + tpos + tvel;
            float Lr = length(tpPV - pPV) / (prad + trad);
            float attr = sc_polar_attr(Lr);
            w += 1.0f;
            dV += (tpPV - pPV) * 0.05f * attr * 1.0f;
            float pap = sc_powf(fminf(1.0f / fmaxf(Lr, 1e-6f), 10.0f) / 10.0f, 0.2f);
            phobSum += pap;
            phobPos += tpPV * pap;
        }
        if (MODE == 0 && (fl & SC_PP_PARTNER)) {
            // dynamics.cuh:584-771: interaction partners, in bond-slot order
            int4 tin = A.info[j];
            const int tid_ = tin.x, ttype = tin.y;
#pragma unroll 1
            for (int k = 0; k < nbi; k++) {
                if (myBonds[3 * k + 2] != tid_) continue;
                const int it = myBonds[3 * k];
                if (it >= 10) {
                    const sc_rule &pii = rule_at(P, it);
                    sc_f4 ro = rule_ori(pii);
                    sc_f3 rp = rule_pos(pii);
                    sc_f4 trot = ld4(A.rotIn, j), tav = ld4(A.avIn, j);
                    sc_f3 tvel = ld3(A.velIn, j);
                    bool o1 = p_order(ptype, pid, ttype, tid_), o2 = p_order(ttype, tid_, ptype, pid);
                    sc_f4 tro_p = o1 ? sc_qmul(trot, sc_qinv(ro)) : sc_qmul(trot, ro);
                    sc_f4 tro_t = o2 ? sc_qmul(prot, sc_qinv(ro)) : sc_qmul(prot, ro);
                    sc_f4 rro = sc_qmul(sc_qinv(sc_qmul(pav, prot)), sc_qmul(tav, tro_p));
                    sc_f4 orro = sc_qmul(sc_qinv(sc_qmul(tav, trot)), sc_qmul(pav, tro_t));
                    dAV = sc_slerp(dAV, sc_qmul(sc_slerp(rro, orro, 0.5f), rro), 0.9f * trad / (prad + trad));
                    sc_f3 rrp = o1 ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(tav, trot)))
                                   : sc_rotate(rp, sc_qmul(tav, trot));
                    rrp += tpos;
                    sc_f3 orrp = o2 ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(pav, prot)))
                                    : sc_rotate(rp, sc_qmul(pav, prot));
                    orrp += ppos;
                    w += 1.0f;
                    sc_f3 pDV = (rrp + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
                    sc_f3 tpDV = (orrp + pvel - (tpos + tvel)) * 0.9f * prad / (prad + trad) * 1.0f;
                    dV += (pDV - (pDV + tpDV) / 2.0f) * 0.9f * prad / (prad + trad) * 1.0f;
                }
                if (it == 0) {
                    if (!dbgTouched) { pdbg = ld4(A.dbg, i); dbgTouched = true; }
                    sc_f4 trot = ld4(A.rotIn, j);
                    bool o1 = p_order(ptype, pid, ttype, tid_);
                    sc_f4 trod = sc_qmul(sc_quat(sc_up(), -SC_PI_REF / 6), sc_quat(sc_right(), SC_PI_REF / 6));
                    prot = sc_slerp(prot, o1 ? sc_qmul(trot, sc_qinv(trod)) : sc_qmul(trot, trod), 0.2f);
                    sc_f4 trpr = sc_quat(sc_forward(), -SC_PI_REF / 6);
                    sc_f3 rrp = o1 ? -sc_rotate(sc_up(), sc_qmul(trot, sc_qmul(sc_qinv(trod), trpr)))
                                   : sc_rotate(sc_up(), sc_qmul(trot, trpr));
                    rrp *= idist;
                    rrp += tpos;
                    pdbg.x = (float)((double)pdbg.x + (double)(rrp.x - ppos.x) * (1.0 - (double)0.2f));
                    pdbg.y = (float)((double)pdbg.y + (double)(rrp.y - ppos.y) * (1.0 - (double)0.2f));
                    pdbg.z = (float)((double)pdbg.z + (double)(rrp.z - ppos.z) * (1.0 - (double)0.2f));
                } else if (it == SC_INTERACTION_TYPE_CHAIN) {
                    if (!dbgTouched) { pdbg = ld4(A.dbg, i); dbgTouched = true; }
                    sc_f3 tvel = ld3(A.velIn, j);
                    sc_f3 nextTup = sc_rotate(sc_rotate(sc_up(), ld4(A.rotIn, j)), pav);
                    sc_f3 nnd = normalize(tpos + tvel - (ppos + pvel));
                    bool fwd = myBonds[3 * k + 1] == SC_INTERACTION_GROUP_FORWARD;
                    dAV = sc_slerp(dAV, sc_quat_from_to(nextUp, (fwd ? -1.0f : 1.0f) * nnd),
                                   0.9f * trad / (prad + trad));
                    sc_f3 relUp = (fwd ? 1.0f : -1.0f) * nextTup;
                    sc_f3 axis = sc_safe_cross(relUp, -nnd);
                    float ang = sc_angle3(relUp, -nnd);
                    sc_f3 rrp = sc_rotate(relUp, sc_quat(axis, fminf(fmaxf(ang, -flex), flex)));
                    rrp *= idist;
                    rrp += tpos;
                    sc_f3 oUp = (fwd ? -1.0f : 1.0f) * nextUp;
                    sc_f3 oaxis = sc_safe_cross(oUp, nnd);
                    float oang = sc_angle3(oUp, nnd);
                    sc_f3 orrp = sc_rotate(oUp, sc_quat(oaxis, fminf(fmaxf(oang, -flex), flex)));
                    orrp *= idist;
                    orrp += ppos;
                    w += 1.0f;
                    sc_f3 pDV = (rrp + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
                    sc_f3 tpDV = (orrp + pvel - (tpos + tvel)) * 0.9f * prad / (prad + trad) * 1.0f;
                    dV += (pDV - (pDV + tpDV) / 2.0f) * 0.9f * prad / (prad + trad) * 1.0f;
                    pdbg.x = (float)((double)pdbg.x + (double)(rrp.x - ppos.x) * (1.0 - (double)0.9f));
                    pdbg.y = (float)((double)pdbg.y + (double)(rrp.y - ppos.y) * (1.0 - (double)0.9f));
                    pdbg.z = (float)((double)pdbg.z + (double)(rrp.z - ppos.z) * (1.0 - (double)0.9f));
                }
            }
        }
        if (fl & SC_PP_COLLIDE) {
            // dynamics.cuh:775-786: soft collision with a non-partner
            sc_f3 nd = normalize(tpos - ppos);
            float cd = prad + trad;
            sc_f3 tvel = ld3(A.velIn, j);
            w += 1.0f;
            dV += (tpos - nd * cd + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
        }
    };
    if (SCAN) {
        BondRegs B;
        B.load(A.nb, A.bonds, i);
        scan27(P, A.cellStart, ppos, reach(P, ppos, P.maxInt, SC_BINNED_P), [&](int j) {
            uint32_t fl = pp_flags(P, IM, i, j, ppos, prad, phydro, B, A.pos, A.info);
            if (fl) body(j, fl);
        });
    } else if (MODE == 2) {
        // plain items list collisions only: the entries, then the
        // neighbours' positions and velocities, of SC_PLAIN_GROUP pairs are
        // loaded together, and the terms added in list order
        const int c = A.L.cnt[i];
        for (int k0 = 0; k0 < c; k0 += SC_PLAIN_GROUP) {
            uint32_t e[SC_PLAIN_GROUP];
            float4 t4[SC_PLAIN_GROUP], tv[SC_PLAIN_GROUP];
#pragma unroll
            for (int q = 0; q < SC_PLAIN_GROUP; q++)
                e[q] = k0 + q < c ? A.L.list[sc_list_at(SC_LIST_PP, i, k0 + q)] : 0u;
#pragma unroll
            for (int q = 0; q < SC_PLAIN_GROUP; q++) {
                t4[q] = make_float4(0, 0, 0, 0);
                tv[q] = t4[q];
                if (k0 + q < c) {
                    const int j = (int)(e[q] & SC_PP_INDEX);
                    t4[q] = A.pos[j];
                    tv[q] = A.velIn[j];
                }
            }
#pragma unroll
            for (int q = 0; q < SC_PLAIN_GROUP; q++) {
                if (k0 + q < c && (e[q] & SC_PP_COLLIDE)) {
                    // dynamics.cuh:775-786
                    const sc_f3 tpos = IM(sc_make_f3(t4[q].x, t4[q].y, t4[q].z));
                    const float trad = t4[q].w;
                    sc_f3 nd = normalize(tpos - ppos);
                    float cd = prad + trad;
                    sc_f3 tvel = sc_make_f3(tv[q].x, tv[q].y, tv[q].z);
                    w += 1.0f;
                    dV += (tpos - nd * cd + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
                }
            }
        }
    } else {
        const int c = A.L.cnt[i];
        for (int k = 0; k < c; k++) {
            uint32_t e = A.L.list[sc_list_at(SC_LIST_PP, i, k)];
            body((int)(e & SC_PP_INDEX), e);
        }
    }
    sc_f3 nv = pvel + dV / fmaxf(w, 1.0f);
    pav = sc_qmul(sc_slerp(sc_qid(), dAV, 1.0f / fmaxf(w, 1.0f)), pav);
    if (phobSum > 0.0f) {
        sc_f3 dir = normalize(phobPos / phobSum - (ppos + nv));
        pav = sc_slerp(pav, sc_quat_from_to(-up, dir), 0.2f);
    }
    st3(A.velOut, i, nv, v4.w);
    st4(A.rotOut, i, prot);
    st4(A.avOut, i, pav);
    if (dbgTouched) st4(A.dbg, i, pdbg);
}

// A plain particle's relaxation (work class 2: collisions only, list path),
// with every load that depends on the item alone already issued by the
// caller (its records, its list count and its first SC_PLAIN_GROUP entries,
// which lie in its list row whatever the count), so the item waits one
// memory latency for them and one more for its neighbours.  The terms are
// relax_item's for this class, in list order.
__device__ __forceinline__ void relax_plain_item(const ScParams &P, const RelaxArgs &A, int i, float4 v4, float4 r4,
                                                 float4 a4, float4 p4, int c, const uint32_t (&e0)[SC_PLAIN_GROUP]) {
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, ppos, SC_BINNED_P);
    const float prad = p4.w;
    const sc_f3 pvel = sc_make_f3(v4.x, v4.y, v4.z);
    sc_f4 pav = sc_make_f4(a4.x, a4.y, a4.z, a4.w);
    sc_f3 dV = sc_zero3();
    const sc_f4 dAV = sc_qid();
    float w = 0.0f;
    uint32_t e[SC_PLAIN_GROUP];
#pragma unroll
    for (int q = 0; q < SC_PLAIN_GROUP; q++) e[q] = e0[q];
    for (int k0 = 0; k0 < c; k0 += SC_PLAIN_GROUP) {
        if (k0 > 0) {
#pragma unroll
            for (int q = 0; q < SC_PLAIN_GROUP; q++)
                e[q] = k0 + q < c ? A.L.list[sc_list_at(SC_LIST_PP, i, k0 + q)] : 0u;
        }
        float4 t4[SC_PLAIN_GROUP], tv[SC_PLAIN_GROUP];
#pragma unroll
        for (int q = 0; q < SC_PLAIN_GROUP; q++) {
            t4[q] = make_float4(0, 0, 0, 0);
            tv[q] = t4[q];
            if (k0 + q < c) {
                const int j = (int)(e[q] & SC_PP_INDEX);
                t4[q] = A.pos[j];
                tv[q] = A.velIn[j];
            }
        }
#pragma unroll
        for (int q = 0; q < SC_PLAIN_GROUP; q++) {
            if (k0 + q < c && (e[q] & SC_PP_COLLIDE)) {
                // dynamics.cuh:775-786
                const sc_f3 tpos = IM(sc_make_f3(t4[q].x, t4[q].y, t4[q].z));
                const float trad = t4[q].w;
                sc_f3 nd = normalize(tpos - ppos);
                float cd = prad + trad;
                sc_f3 tvel = sc_make_f3(tv[q].x, tv[q].y, tv[q].z);
                w += 1.0f;
                dV += (tpos - nd * cd + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
            }
        }
    }
    sc_f3 nv = pvel + dV / fmaxf(w, 1.0f);
    pav = sc_qmul(sc_slerp(sc_qid(), dAV, 1.0f / fmaxf(w, 1.0f)), pav);
    st3(A.velOut, i, nv, v4.w);
    A.rotOut[i] = r4;
    st4(A.avOut, i, pav);
}

// A polar particle's relaxation (work class 1: polar and collision pairs,
// list path): relax_item's terms for this class in list order, with the
// entries of SC_POLAR_GROUP pairs, then their neighbours' positions,
// velocities and (polar pairs) rotations, loaded together.
#define SC_POLAR_GROUP 2
__device__ __forceinline__ void relax_polar_item(const ScParams &P, const RelaxArgs &A, int i, int4 in, float4 v4,
                                                 float4 r4, float4 a4, float4 p4, int c) {
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, ppos, SC_BINNED_P);
    const float prad = p4.w;
    const sc_f3 pvel = sc_make_f3(v4.x, v4.y, v4.z);
    const sc_f4 prot = sc_make_f4(r4.x, r4.y, r4.z, r4.w);
    sc_f4 pav = sc_make_f4(a4.x, a4.y, a4.z, a4.w);
    const int phydro = (int)(int8_t)(in.w & 0xff);
    (void)phydro;
    sc_f3 dV = sc_zero3();
    const sc_f4 dAV = sc_qid();
    sc_f3 phobPos = sc_zero3();
    float phobSum = 0.0f;
    float w = 0.0f;
    const sc_f3 up = sc_rotate(sc_up(), prot);
    const sc_f3 nextUp = sc_rotate(up, pav);
    for (int k0 = 0; k0 < c; k0 += SC_POLAR_GROUP) {
        uint32_t e[SC_POLAR_GROUP];
#pragma unroll
        for (int q = 0; q < SC_POLAR_GROUP; q++) e[q] = k0 + q < c ? A.L.list[sc_list_at(SC_LIST_PP, i, k0 + q)] : 0u;
        float4 t4[SC_POLAR_GROUP], tv[SC_POLAR_GROUP], tr[SC_POLAR_GROUP];
#pragma unroll
        for (int q = 0; q < SC_POLAR_GROUP; q++) {
            t4[q] = make_float4(0, 0, 0, 0);
            tv[q] = t4[q];
            tr[q] = t4[q];
            if (k0 + q < c) {
                const int j = (int)(e[q] & SC_PP_INDEX);
                t4[q] = A.pos[j];
                if (e[q] & (SC_PP_POLAR | SC_PP_COLLIDE)) tv[q] = A.velIn[j];
                if (e[q] & SC_PP_POLAR) tr[q] = A.rotIn[j];
            }
        }
#pragma unroll
        for (int q = 0; q < SC_POLAR_GROUP; q++) {
            if (k0 + q >= c) break;
            const uint32_t fl = e[q];
            const sc_f3 tpos = IM(sc_make_f3(t4[q].x, t4[q].y, t4[q].z));
            const float trad = t4[q].w;
            const sc_f3 tvel = sc_make_f3(tv[q].x, tv[q].y, tv[q].z);
            if (fl & SC_PP_POLAR) {
                // dynamics.cuh:478-582: polar (lipid) head / tail attraction
                sc_f3 nextTup = sc_rotate(sc_rotate(sc_up(), sc_make_f4(tr[q].x, tr[q].y, tr[q].z, tr[q].w)), pav);
                sc_f3 pPV = -nextUp * prad + ppos + pvel;
                sc_f3 tpPV = -nextTup * trad + tpos + tvel;
                float Lr = length(tpPV - pPV) / (prad + trad);
                float attr = sc_polar_attr(Lr);
                w += 1.0f;
                dV += (tpPV - pPV) * 0.05f * attr * 1.0f;
                float pap = sc_powf(fminf(1.0f / fmaxf(Lr, 1e-6f), 10.0f) / 10.0f, 0.2f);
                phobSum += pap;
                phobPos += tpPV * pap;
            }
            if (fl & SC_PP_COLLIDE) {
                // dynamics.cuh:775-786: soft collision with a non-partner
                sc_f3 nd = normalize(tpos - ppos);
                float cd = prad + trad;
                w += 1.0f;
                dV += (tpos - nd * cd + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
            }
        }
    }
    sc_f3 nv = pvel + dV / fmaxf(w, 1.0f);
    pav = sc_qmul(sc_slerp(sc_qid(), dAV, 1.0f / fmaxf(w, 1.0f)), pav);
    if (phobSum > 0.0f) {
        sc_f3 dir = normalize(phobPos / phobSum - (ppos + nv));
        pav = sc_slerp(pav, sc_quat_from_to(-up, dir), 0.2f);
    }
    st3(A.velOut, i, nv, v4.w);
    A.rotOut[i] = r4;
    st4(A.avOut, i, pav);
}

// A bonded particle's relaxation (work class 0, list path).  The pose terms
// of its rule and chain bonds do not depend on the running sums, so they are
// evaluated first, from its bond matches (k_build_pp records them in the
// order the reference meets them), with every lane of a warp on its own
// first bond, then its second ...; the list is then walked once more to add
// every term in the reference's order (the slerps of dAV and the float sums
// are order-dependent).  A test bond rotates the particle itself, which
// later terms read: such particles (SC_MATCH_INORDER) take the in-order
// scan of k_relax_overflow.
struct BondTerm {
    sc_f3 dv;   // velocity term
    sc_f4 q;    // dAV slerp target
    float t;    // dAV slerp weight
    sc_f3 dbg;  // chain bonds: rrp - ppos for the debug vector
};

__device__ __forceinline__ void relax_bonded_item(const ScParams &P, const RelaxArgs &A, int i, int4 in, float4 v4,
                                                  float4 r4, float4 a4) {
    const int *__restrict__ myBonds = A.bonds + (size_t)i * 24;
    float4 p4 = A.pos[i];
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, ppos, SC_BINNED_P);
    const float prad = p4.w;
    const sc_f3 pvel = sc_make_f3(v4.x, v4.y, v4.z);
    const sc_f4 prot = sc_make_f4(r4.x, r4.y, r4.z, r4.w);
    sc_f4 pav = sc_make_f4(a4.x, a4.y, a4.z, a4.w);
    const int pid = in.x, ptype = in.y;
    const sc_f3 up = sc_rotate(sc_up(), prot);
    const sc_f3 nextUp = sc_rotate(up, pav);
    const float flex = SC_PI_REF / 8;
    const int c = A.L.cnt[i];
    // 1. the terms of its bond matches (list order, then bond-slot order)
    const uint32_t *__restrict__ myMatch = A.match + (size_t)i * SC_MAX_ACTIVE_INTERACTIONS;
    const int nm = min(A.matchN[i] & SC_MATCH_COUNT, SC_MAX_ACTIVE_INTERACTIONS);
    // the first term stays in registers (most bonded items have one); the
    // rest go to a per-thread array
    BondTerm T0, T[SC_MAX_ACTIVE_INTERACTIONS - 1];
    int nt = 0;
    for (int m = 0; m < nm; m++) {
        const uint32_t me = myMatch[m];
        const int j = (int)(me & SC_PP_INDEX), k = (int)(me >> 29);
        const int it = myBonds[3 * k];
        if (!(it >= 10 || it == SC_INTERACTION_TYPE_CHAIN) || nt >= SC_MAX_ACTIVE_INTERACTIONS) continue;
        const int4 tin = A.info[j];
        const int tid_ = tin.x, ttype = tin.y;
        const float4 t4 = A.pos[j];
        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
        const float trad = t4.w, idist = prad + trad;
        const sc_f4 trot = ld4(A.rotIn, j), tav = ld4(A.avIn, j);
        const sc_f3 tvel = ld3(A.velIn, j);
        BondTerm b;
        if (it >= 10) {
            // dynamics.cuh:591-655
            const sc_rule &pii = rule_at(P, it);
            sc_f4 ro = rule_ori(pii);
            sc_f3 rp = rule_pos(pii);
            bool o1 = p_order(ptype, pid, ttype, tid_), o2 = p_order(ttype, tid_, ptype, pid);
            sc_f4 tro_p = o1 ? sc_qmul(trot, sc_qinv(ro)) : sc_qmul(trot, ro);
            sc_f4 tro_t = o2 ? sc_qmul(prot, sc_qinv(ro)) : sc_qmul(prot, ro);
            sc_f4 rro = sc_qmul(sc_qinv(sc_qmul(pav, prot)), sc_qmul(tav, tro_p));
            sc_f4 orro = sc_qmul(sc_qinv(sc_qmul(tav, trot)), sc_qmul(pav, tro_t));
            b.q = sc_qmul(sc_slerp(rro, orro, 0.5f), rro);
            b.t = 0.9f * trad / (prad + trad);
            sc_f3 rrp = o1 ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(tav, trot))) : sc_rotate(rp, sc_qmul(tav, trot));
            rrp += tpos;
            sc_f3 orrp = o2 ? sc_rotate(-rp, sc_qmul(sc_qinv(ro), sc_qmul(pav, prot))) : sc_rotate(rp, sc_qmul(pav, prot));
            orrp += ppos;
            sc_f3 pDV = (rrp + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
            sc_f3 tpDV = (orrp + pvel - (tpos + tvel)) * 0.9f * prad / (prad + trad) * 1.0f;
            b.dv = (pDV - (pDV + tpDV) / 2.0f) * 0.9f * prad / (prad + trad) * 1.0f;
        } else {
            // dynamics.cuh:692-769
            sc_f3 nextTup = sc_rotate(sc_rotate(sc_up(), trot), pav);
            sc_f3 nnd = normalize(tpos + tvel - (ppos + pvel));
            bool fwd = myBonds[3 * k + 1] == SC_INTERACTION_GROUP_FORWARD;
            b.q = sc_quat_from_to(nextUp, (fwd ? -1.0f : 1.0f) * nnd);
            b.t = 0.9f * trad / (prad + trad);
            sc_f3 relUp = (fwd ? 1.0f : -1.0f) * nextTup;
            sc_f3 axis = sc_safe_cross(relUp, -nnd);
            float ang = sc_angle3(relUp, -nnd);
            sc_f3 rrp = sc_rotate(relUp, sc_quat(axis, fminf(fmaxf(ang, -flex), flex)));
            rrp *= idist;
            rrp += tpos;
            sc_f3 oUp = (fwd ? -1.0f : 1.0f) * nextUp;
            sc_f3 oaxis = sc_safe_cross(oUp, nnd);
            float oang = sc_angle3(oUp, nnd);
            sc_f3 orrp = sc_rotate(oUp, sc_quat(oaxis, fminf(fmaxf(oang, -flex), flex)));
            orrp *= idist;
            orrp += ppos;
            sc_f3 pDV = (rrp + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
            sc_f3 tpDV = (orrp + pvel - (tpos + tvel)) * 0.9f * prad / (prad + trad) * 1.0f;
            b.dv = (pDV - (pDV + tpDV) / 2.0f) * 0.9f * prad / (prad + trad) * 1.0f;
            b.dbg = rrp - ppos;
        }
        if (nt == 0)
            T0 = b;
        else
            T[nt - 1] = b;
        nt++;
    }
    // 3. every term in the reference's order
    sc_f4 pdbg = sc_make_f4(0, 0, 0, 0);
    bool dbgTouched = false;
    sc_f3 dV = sc_zero3();
    sc_f4 dAV = sc_qid();
    sc_f3 phobPos = sc_zero3();
    float phobSum = 0.0f;
    float w = 0.0f;
    int ut = 0, mi = 0;
    for (int kk = 0; kk < c; kk++) {
        const uint32_t fl = A.L.list[sc_list_at(SC_LIST_PP, i, kk)];
        const int j = (int)(fl & SC_PP_INDEX);
        float4 t4 = A.pos[j];
        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
        const float trad = t4.w;
        if (fl & SC_PP_POLAR) {
            sc_f3 tvel = ld3(A.velIn, j);
            sc_f3 nextTup = sc_rotate(sc_rotate(sc_up(), ld4(A.rotIn, j)), pav);
            sc_f3 pPV = -nextUp * prad + ppos + pvel;
            sc_f3 tpPV = -nextTup * trad + tpos + tvel;
            float Lr = length(tpPV - pPV) / (prad + trad);
            float attr = sc_polar_attr(Lr);
            w += 1.0f;
            dV += (tpPV - pPV) * 0.05f * attr * 1.0f;
            float pap = sc_powf(fminf(1.0f / fmaxf(Lr, 1e-6f), 10.0f) / 10.0f, 0.2f);
            phobSum += pap;
            phobPos += tpPV * pap;
        }
        if (fl & SC_PP_PARTNER) {
            // this neighbour's bond matches are the next ones in order
            for (; mi < nm && (int)(myMatch[mi] & SC_PP_INDEX) == j; mi++) {
                const int k = (int)(myMatch[mi] >> 29);
                const int it = myBonds[3 * k];
                if ((it >= 10 || it == SC_INTERACTION_TYPE_CHAIN) && ut < nt) {
                    const BondTerm b = ut == 0 ? T0 : T[ut - 1];
                    ut++;
                    if (it == SC_INTERACTION_TYPE_CHAIN && !dbgTouched) {
                        pdbg = ld4(A.dbg, i);
                        dbgTouched = true;
                    }
                    dAV = sc_slerp(dAV, b.q, b.t);
                    w += 1.0f;
                    dV += b.dv;
                    if (it == SC_INTERACTION_TYPE_CHAIN) {
                        pdbg.x = (float)((double)pdbg.x + (double)b.dbg.x * (1.0 - (double)0.9f));
                        pdbg.y = (float)((double)pdbg.y + (double)b.dbg.y * (1.0 - (double)0.9f));
                        pdbg.z = (float)((double)pdbg.z + (double)b.dbg.z * (1.0 - (double)0.9f));
                    }
                }
            }
        }
        if (fl & SC_PP_COLLIDE) {
            sc_f3 nd = normalize(tpos - ppos);
            float cd = prad + trad;
            sc_f3 tvel = ld3(A.velIn, j);
            w += 1.0f;
            dV += (tpos - nd * cd + tvel - (ppos + pvel)) * 0.9f * trad / (prad + trad) * 1.0f;
        }
    }
    sc_f3 nv = pvel + dV / fmaxf(w, 1.0f);
    pav = sc_qmul(sc_slerp(sc_qid(), dAV, 1.0f / fmaxf(w, 1.0f)), pav);
    if (phobSum > 0.0f) {
        sc_f3 dir = normalize(phobPos / phobSum - (ppos + nv));
        pav = sc_slerp(pav, sc_quat_from_to(-up, dir), 0.2f);
    }
    st3(A.velOut, i, nv, v4.w);
    st4(A.rotOut, i, prot);
    st4(A.avOut, i, pav);
    if (dbgTouched) st4(A.dbg, i, pdbg);
}

// One item of a work class (the items whose list overflowed, and bonded
// items with a test bond, are left to k_relax_overflow).
template <int MODE, bool BATCH>
__device__ __forceinline__ void relax_class_item(const ScParams &P0, const RelaxArgs &A, int i) {
    if (MODE == 2) {
        const int4 in = A.info[i];
        const float4 v4 = A.velIn[i], r4 = A.rotIn[i], a4 = A.avIn[i], p4 = A.pos[i];
        const int c = A.L.cnt[i];
        uint32_t e0[SC_PLAIN_GROUP];
#pragma unroll
        for (int q = 0; q < SC_PLAIN_GROUP; q++) e0[q] = A.L.list[sc_list_at(SC_LIST_PP, i, q)];
        if (!(in.z & SC_ACTIVE)) {
            A.velOut[i] = v4;
            A.rotOut[i] = r4;
            A.avOut[i] = a4;
            return;
        }
        ScParams P = P0;
        rep_apply<BATCH>(P, in.w);
        if (c > min(SC_LIST_PP, P.listLimit)) return;
        relax_plain_item(P, A, i, v4, r4, a4, p4, c, e0);
        return;
    }
    int4 in = A.info[i];
    float4 v4 = A.velIn[i], r4 = A.rotIn[i], a4 = A.avIn[i];
    if (!(in.z & SC_ACTIVE)) {
        A.velOut[i] = v4;
        A.rotOut[i] = r4;
        A.avOut[i] = a4;
        return;
    }
    ScParams P = P0;
    rep_apply<BATCH>(P, in.w);
    if (A.L.cnt[i] > min(SC_LIST_PP, P.listLimit)) return;
    if (MODE == 0) {
        if (!(A.matchN[i] & SC_MATCH_INORDER)) relax_bonded_item(P, A, i, in, v4, r4, a4);
    } else {
        relax_polar_item(P, A, i, in, v4, r4, a4, A.pos[i], A.L.cnt[i]);
    }
}

// The items of one work class, grid-stride over the class's index segment.
// The bonded class goes block by block, its items ranked by bond-match
// count (chain-bonded apart from rule-bonded) inside the block, so a warp's
// lanes walk about as many bond terms of the same kind (items with more
// bonds would otherwise hold back the rest of their warp).
template <int MODE, bool BATCH>
__global__ void __launch_bounds__(SC_THREADS, MODE == 0 ? 2 : 4) k_relax(ScParams P, RelaxArgs A) {
    const int n = A.classCount[MODE];
    const int *__restrict__ idx = A.classIdx + (size_t)MODE * A.L.cap;
    if (MODE == 0) {
        __shared__ int s_item[SC_THREADS];
        for (int base = blockIdx.x * SC_THREADS; base < n; base += gridDim.x * SC_THREADS) {
            const int t = base + threadIdx.x;
            const int i = t < n ? idx[t] : -1;
            s_item[threadIdx.x] = i;
            // rank key: bond-match count, chain-bonded items apart from rule-bonded ones (their
            // pose terms are different code)
            int key = 0;
            if (i >= 0)
                key = (A.matchN[i] & SC_MATCH_COUNT) +
                      (A.bonds[(size_t)i * 24] == SC_INTERACTION_TYPE_CHAIN ? SC_MAX_ACTIVE_INTERACTIONS + 1 : 0);
            int src, cs;
            count_rank<2 * SC_MAX_ACTIVE_INTERACTIONS + 1>(i >= 0, key, &src, &cs);
            if (cs >= 0) relax_class_item<MODE, BATCH>(P, A, s_item[src]);
            __syncthreads();  // the ranking's shared arrays are reused by the next round
        }
    } else {
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
            relax_class_item<MODE, BATCH>(P, A, idx[t]);
    }
}

// Active items whose list overflowed: their neighbourhood is scanned.  A
// separate kernel keeps the scan code out of k_relax's instruction stream.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_relax_overflow(ScParams P, RelaxArgs A, const int *__restrict__ ovf,
                                                               const int *__restrict__ ovfCount) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *ovfCount; t += gridDim.x * blockDim.x) {
        const int i = ovf[t];
        int4 in = A.info[i];
        rep_apply<BATCH>(P, in.w);
        if (in.z & SC_ACTIVE) relax_item<true, 0>(P, A, i, in, A.velIn[i], A.rotIn[i], A.avIn[i]);
    }
}

// (float)((double)(rp + rt) + 0.8 * (double)rp) (metabolites.cuh:198,237,324),
// recomputed only when the partner radius changes.
struct CollisionDistCache {
    float rt = 0.0f, cd = 0.0f;
    sc_sqrt_le le;
    bool valid = false;
    __device__ __forceinline__ float get(float rp, float r) {
        if (!valid || !(r == rt)) {
            rt = r;
            valid = true;
            cd = sc_coll_dist(rp, r);
            le = sc_sqrt_le_make(cd);
        }
        return cd;
    }
    // sc_norm3(delta) <= the collision distance of (rp, r), the reference's
    // test (metabolites.cuh:193-203), mostly without the square root
    __device__ __forceinline__ bool collides(float rp, float r, sc_f3 delta) {
        get(rp, r);
        return sc_sqrt_le_test(le, sc_normsq3(delta));
    }
};

// ---- metabolites.cuh:140-264 relaxMetabolicParticles ----------------------
// List: per metabolic item, cell by cell, the colliding metabolic items then
// the colliding lipids (SC_M_FROM_P), as the reference's loops visit them.
// The M list of metabolic item i, written at position i of `list`.
// The colliding metabolic items, then lipids, of each neighbour cell of
// metabolic item i in visiting order, each handed to sink(j, fromP, t4) (j
// the neighbour's slot, t4 its position and radius; the collision distance is
// then cached in cm / cp).
template <class Sink>
__device__ __forceinline__ void scan_m_item(const ScParams &P, const uint32_t *__restrict__ cellStartM,
                                            const uint32_t *__restrict__ cellStartP, int i,
                                            const float4 *__restrict__ mpos, const int4 *__restrict__ minfo,
                                            const float4 *__restrict__ ppos_, const int4 *__restrict__ pinfo,
                                            const Imager &IM, sc_f3 pp, float prad, CollisionDistCache &cm,
                                            CollisionDistCache &cp, Sink &&sink) {
    const float lim = P.maxInt;
    cells27(P, pp, reach(P, pp, lim, SC_BINNED_M | SC_BINNED_P), [&](uint32_t key) {
        for (uint32_t j = cellStartM[key], e = cellStartM[key + 1]; j < e; j++) {
            if ((int)j == i || !active_m(P, minfo, (int)j)) continue;
            float4 t4 = mpos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) continue;
            if (cm.collides(prad, t4.w, delta)) sink(j, false, t4);
        }
        for (uint32_t j = cellStartP[key], e = cellStartP[key + 1]; j < e; j++) {
            if (!active_lipid(P, pinfo, (int)j)) continue;
            float4 t4 = ppos_[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) continue;
            if (cp.collides(prad, t4.w, delta)) sink(j, true, t4);
        }
    });
}

__device__ __forceinline__ void build_m_item(const ScParams &P, const uint32_t *__restrict__ cellStartM,
                                             const uint32_t *__restrict__ cellStartP, int i,
                                             const float4 *__restrict__ mpos, const int4 *__restrict__ minfo,
                                             const float4 *__restrict__ ppos_, const int4 *__restrict__ pinfo,
                                             uint32_t *list, int &c) {
    float4 p4 = mpos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
    CollisionDistCache cm, cp;
    const int limit = min(SC_LIST_M, P.listLimit);
    scan_m_item(P, cellStartM, cellStartP, i, mpos, minfo, ppos_, pinfo, IM, pp, p4.w, cm, cp,
                [&](uint32_t j, bool fromP, float4) {
                    if (c < limit) list[sc_list_at(SC_LIST_M, i, c)] = fromP ? (j | SC_M_FROM_P) : j;
                    c++;
                });
}

// The full pair lists of the metabolic items whose list overflowed (listed
// by k_build_m with their pair counts): each takes a contiguous region of
// the overflow pool by atomicAdd and writes its pairs there in visiting order,
// 16-byte entries with the frozen geometry as the main pool's; an item the
// pool has no room for keeps offset -1 (it scans its neighbourhood).  The
// demand is counted in full for the pool's growth at the next synchronisation.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_m_ovf(
    ScParams P0, const uint32_t *__restrict__ cellStartM, const uint32_t *__restrict__ cellStartP,
    const float4 *__restrict__ mpos, const int4 *__restrict__ minfo, const float4 *__restrict__ ppos_,
    const int4 *__restrict__ pinfo, const int *__restrict__ ovf, const int *__restrict__ ovfCount,
    const int *__restrict__ ovfN, long long *__restrict__ ovfOff, uint4 *__restrict__ pool, long long cap,
    unsigned long long *__restrict__ demand) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *ovfCount; t += gridDim.x * blockDim.x) {
        const int i = ovf[t], n = ovfN[t];
        const unsigned long long base = n > 0 ? atomicAdd(demand, (unsigned long long)n) : 0ull;
        if (n <= 0 || base + (unsigned long long)n > (unsigned long long)cap) {
            ovfOff[t] = -1;
            continue;
        }
        ovfOff[t] = (long long)base;
        ScParams P = P0;
        rep_apply<BATCH>(P, minfo[i].w);
        const float4 p4 = mpos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
        const float prad = p4.w;
        CollisionDistCache cm, cp;
        uint4 *out = pool + base;
        int k = 0;
        scan_m_item(P, cellStartM, cellStartP, i, mpos, minfo, ppos_, pinfo, IM, pp, prad, cm, cp,
                    [&](uint32_t j, bool fromP, float4 t4) {
                        if (k >= n) return;
                        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
                        const sc_f3 nd = normalize(tpos - pp);
                        const float cd = fromP ? cp.get(prad, t4.w) : cm.get(prad, t4.w);
                        const sc_f3 a = tpos - nd * cd;
                        out[k++] = make_uint4(fromP ? (j | SC_M_FROM_P) : j, __float_as_uint(a.x),
                                              __float_as_uint(a.y), __float_as_uint(a.z));
                    });
    }
}

// A pool position for the pairs of one count-ordered list position: the
// block's items are ranked by count, each warp takes a region of
// (its longest list) x 32 entries of the pool, and a list that does not fit
// its capacity, or every list of a block the pool has no room for, is marked
// overflowed (cnt = INT_MAX; listed in `ovf` when given).  Returns the item,
// how many pairs to write and where its first one goes (entry k at
// out[32 k]).  With `items`, thread t of the block stands for item
// items[b0 + t] (a compacted list) and perm holds those items.
template <class T>
struct PoolSlot {
    int i, n;
    T *out;
};
template <int K, class T>
__device__ __forceinline__ PoolSlot<T> pool_take(const ScParams &P, bool valid, int c, T *__restrict__ pool,
                                              long long poolCap, unsigned long long *__restrict__ poolUsed, long long *__restrict__ warpOff,
                                              int *__restrict__ cnt, int *__restrict__ perm, int cap,
                                              int *__restrict__ ovf, int *__restrict__ ovfCount,
                                              const int *__restrict__ items = nullptr, int *__restrict__ ovfN = nullptr) {
    __shared__ int s_n[SC_THREADS / 32];
    __shared__ long long s_base;
    const int b0 = blockIdx.x * SC_THREADS, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int src, cs;
    count_rank<K>(valid, c, &src, &cs);
    const int limit = min(K, P.listLimit);
    bool ovfl = cs > limit;
    int n = ovfl ? 0 : max(cs, 0);
    // the warp's longest stored list (overflowed lists rank first but store nothing)
    const int wmax = __reduce_max_sync(0xffffffffu, n);
    if (lane == 0) s_n[warp] = wmax;
    __syncthreads();
    if (t == 0) {
        int total = 0;
        for (int w = 0; w < SC_THREADS / 32; w++) total += s_n[w] * 32;
        // 64-bit demand: it keeps counting what blocks ask for past the pool
        const unsigned long long base = total ? atomicAdd(poolUsed, (unsigned long long)total) : 0ull;
        s_base = base + (unsigned long long)total <= (unsigned long long)poolCap ? (long long)base : -1ll;
    }
    __syncthreads();
    if (s_base < 0 && cs > 0) {
        ovfl = true;
        n = 0;
    }
    long long off = s_base;
    for (int w = 0; w < warp; w++) off += s_n[w] * 32;
    const int g = b0 + t;
    if (g < cap) {
        perm[g] = cs >= 0 ? (items ? items[b0 + src] : b0 + src) : -1;
        cnt[g] = ovfl ? INT_MAX : max(cs, 0);
        if (lane == 0) warpOff[g >> 5] = s_base < 0 ? 0 : off;
    }
    if (ovfl && ovf) {
        const int t = atomicAdd(ovfCount, 1);
        ovf[t] = b0 + src;
        if (ovfN) ovfN[t] = max(cs, 0);  // its full pair count
    }
    PoolSlot<T> r;
    r.i = cs >= 0 && items ? items[b0 + src] : b0 + src;
    r.n = n;
    r.out = pool + (n ? off : 0) + lane;
    return r;
}

// M pairs with their frozen geometry.  Positions do not change between the
// sort and applyVelocities, so for every listed pair the part of the
// reference's velocity term that depends on positions only,
// A = tpos - normalize(tpos - pos) * collisionDistance (metabolites.cuh:
// 196-203, 235-242), is the same in every relaxation sub-iteration.  It is
// evaluated here, once per step, and each sub-iteration adds
// ((A + tvel) - (pos + vel)) * 0.9 * weight: A is exactly the float3 the
// reference's expression evaluates first, so sums and rounding are its own.
// Layout: the pairs of a warp's 32 positions share one region of the pool,
// entry k of lane l at warpOff[w] + 32 k + l, 16 bytes {neighbour | kind,
// A.x, A.y, A.z}; a region is sized by the warp's longest stored list.  An
// overflowed item, or every item of a block the pool has no room for, is
// listed in `ovf` for the scan.
template <bool BATCH>
__device__ __forceinline__ void emit_m_pairs(const ScParams &P0, bool valid, int c, const uint32_t *scratch,
                                             const int4 *__restrict__ minfo,
                                             const float4 *__restrict__ mpos, const float4 *__restrict__ ppos_,
                                             uint4 *__restrict__ pool, long long poolCap, unsigned long long *__restrict__ poolUsed,
                                             long long *__restrict__ warpOff, int *__restrict__ cnt, int *__restrict__ perm,
                                             int cap, int *__restrict__ ovf, int *__restrict__ ovfCount,
                                             int *__restrict__ ovfN) {
    const PoolSlot<uint4> S = pool_take<SC_LIST_M>(P0, valid, c, pool, poolCap, poolUsed, warpOff, cnt, perm, cap, ovf,
                                                   ovfCount, nullptr, ovfN);
    if (S.n == 0) return;
    const int i = S.i;
    ScParams P = P0;
    rep_apply<BATCH>(P, minfo[i].w);
    const float4 p4 = mpos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
    const float prad = p4.w;
    CollisionDistCache cm, cp;
    for (int k = 0; k < S.n; k++) {
        const uint32_t e = scratch[sc_list_at(SC_LIST_M, i, k)];
        const int j = (int)(e & SC_M_INDEX);
        const bool fromP = (e & SC_M_FROM_P) != 0;
        const float4 t4 = fromP ? ppos_[j] : mpos[j];
        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
        const sc_f3 nd = normalize(tpos - pp);
        const float cd = fromP ? cp.get(prad, t4.w) : cm.get(prad, t4.w);
        const sc_f3 a = tpos - nd * cd;
        S.out[(size_t)k * 32] = make_uint4(e, __float_as_uint(a.x), __float_as_uint(a.y), __float_as_uint(a.z));
    }
}

// The lean form of the same pool (ScParams.metabLean): 4-byte entries
// {neighbour | kind} only, in the same count-ordered warp regions; the
// relaxation re-evaluates the geometry from the neighbour's position each
// sub-iteration (a 16-byte gather that nearby items share in L1 / L2, and a
// square root and a division per pair) instead of streaming 12 more bytes
// per pair from HBM.
__device__ __forceinline__ void emit_m_pairs_lean(const ScParams &P, bool valid, int c, const uint32_t *scratch,
                                                  uint32_t *__restrict__ pool, long long poolCap,
                                                  unsigned long long *__restrict__ poolUsed, long long *__restrict__ warpOff,
                                                  int *__restrict__ cnt, int *__restrict__ perm, int cap,
                                                  int *__restrict__ ovf, int *__restrict__ ovfCount,
                                                  int *__restrict__ ovfN) {
    const PoolSlot<uint32_t> S = pool_take<SC_LIST_M>(P, valid, c, pool, poolCap, poolUsed, warpOff, cnt, perm, cap,
                                                      ovf, ovfCount, nullptr, ovfN);
    for (int k = 0; k < S.n; k++) S.out[(size_t)k * 32] = scratch[sc_list_at(SC_LIST_M, S.i, k)];
}

template <bool LEAN, bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_m(ScParams P0, const uint32_t *__restrict__ cellStartM,
                                                        const uint32_t *__restrict__ cellStartP,
                                                        const int *__restrict__ nActivePtr,
                                                        const float4 *__restrict__ mpos, const int4 *__restrict__ minfo,
                                                        const float4 *__restrict__ ppos_, const int4 *__restrict__ pinfo,
                                                        uint32_t *__restrict__ pool, long long poolCap,
                                                        unsigned long long *__restrict__ poolUsed,
                                                        long long *__restrict__ warpOff, uint32_t *scratch,
                                                        int *__restrict__ cnt, int *__restrict__ perm, int cap,
                                                        int *__restrict__ ovf, int *__restrict__ ovfCount,
                                                        int *__restrict__ ovfN) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < *nActivePtr;
    int c = 0;
    if (valid) {
        const int4 mi = minfo[i];
        ScParams P = P0;
        rep_apply<BATCH>(P, mi.w);
        if (mi.z & SC_ACTIVE) build_m_item(P, cellStartM, cellStartP, i, mpos, minfo, ppos_, pinfo, scratch, c);
    }
    if (LEAN)
        emit_m_pairs_lean(P0, valid, c, scratch, pool, poolCap, poolUsed, warpOff, cnt, perm, cap, ovf, ovfCount, ovfN);
    else
        emit_m_pairs<BATCH>(P0, valid, c, scratch, minfo, mpos, ppos_, reinterpret_cast<uint4 *>(pool), poolCap,
                            poolUsed, warpOff, cnt, perm, cap, ovf, ovfCount, ovfN);
}


struct RelaxMArgs {
    const uint32_t *__restrict__ cellStartM, *__restrict__ cellStartP;
    const int *__restrict__ nActivePtr;
    const float4 *__restrict__ mpos;
    const int4 *__restrict__ minfo;
    PairList<SC_LIST_M> L;
    const float4 *__restrict__ mvelIn;
    float4 *__restrict__ mvelOut;
    const float4 *__restrict__ ppos;
    const int4 *__restrict__ pinfo;
    const float4 *__restrict__ pvel;
    const uint4 *__restrict__ pool;     // pairs with their geometry (emit_m_pairs)
    const long long *__restrict__ warpOff;
};

// The contribution of one colliding neighbour (a metabolic item, or a lipid
// with twice the weight) to dV and w, metabolites.cuh:196-203 / 235-242.
__device__ __forceinline__ void metab_pair(const Imager &IM, sc_f3 pp, sc_f3 ppv, float4 t4, float4 tv, float cd,
                                           bool fromP, sc_f3 &dV, float &w) {
    sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
    sc_f3 nd = normalize(tpos - pp);
    float k = fromP ? 2.0f : 1.0f;
    w += k;
    dV += (tpos - nd * cd + sc_make_f3(tv.x, tv.y, tv.z) - ppv) * 0.9f * k;
}

// One pair's neighbour velocity: a metabolic item's, or a lipid's.
__device__ __forceinline__ float4 metab_pair_vel(const RelaxMArgs &A, uint32_t e) {
    return ((e & SC_M_FROM_P) ? A.pvel : A.mvelIn)[e & SC_M_INDEX];
}

// Items whose list fits, in count order: each pair adds its precomputed
// geometry and the neighbour's current velocity, in list order.  Pairs are
// taken SC_METAB_GROUP at a time: the group's neighbour velocities and the
// next group's entries are all in flight together, so a thread waits about
// one memory latency per group instead of one per pair.  Entries are read
// once per launch (evict-first); velocities are re-read by nearby items.
#define SC_METAB_GROUP 4
__global__ void __launch_bounds__(SC_THREADS, 4) k_relax_metab(ScParams P, RelaxMArgs A) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;   // list position (count-ordered)
    if (g >= *A.nActivePtr) return;
    const int i = A.L.perm[g];
    if (i < 0) return;
    const float4 v4 = A.mvelIn[i];
    // after the sort the active items are exactly the binned ones
    const bool act = P.mAllActive ? i < (int)A.cellStartM[P.cells] : (A.minfo[i].z & SC_ACTIVE) != 0;
    if (!act) {
        A.mvelOut[i] = v4;
        return;
    }
    const int c = A.L.cnt[g];
    if (c > min(SC_LIST_M, P.listLimit)) return;
    const float4 p4 = A.mpos[i];
    const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
    const sc_f3 ppv = sc_make_f3(p4.x, p4.y, p4.z) + pv;
    sc_f3 dV = sc_zero3();
    float w = 0.0f;
    const uint4 *pairs = A.pool + A.warpOff[g >> 5] + (g & 31);
    uint4 E[SC_METAB_GROUP];
#pragma unroll
    for (int q = 0; q < SC_METAB_GROUP; q++) E[q] = q < c ? __ldcs(pairs + (size_t)q * 32) : make_uint4(0, 0, 0, 0);
    for (int k0 = 0; k0 < c; k0 += SC_METAB_GROUP) {
        float4 tv[SC_METAB_GROUP];
        uint4 En[SC_METAB_GROUP];
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) tv[q] = k0 + q < c ? metab_pair_vel(A, E[q].x) : make_float4(0, 0, 0, 0);
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) {
            const int k = k0 + SC_METAB_GROUP + q;
            En[q] = k < c ? __ldcs(pairs + (size_t)k * 32) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) {
            if (k0 + q < c) {
                const float kw = (E[q].x & SC_M_FROM_P) ? 2.0f : 1.0f;
                const sc_f3 a = sc_make_f3(__uint_as_float(E[q].y), __uint_as_float(E[q].z), __uint_as_float(E[q].w));
                w += kw;
                dV += (a + sc_make_f3(tv[q].x, tv[q].y, tv[q].z) - ppv) * 0.9f * kw;
            }
            E[q] = En[q];
        }
    }
    st3(A.mvelOut, i, pv + dV / fmaxf(w, 1.0f), v4.w);
}

// The lean pool's sweep: per pair the neighbour's position and velocity are
// gathered and the reference's term (metab_pair) evaluated in full, pairs
// taken SC_METAB_GROUP at a time as in k_relax_metab.  The image test of a
// periodic box is decided once per item (Imager), the collision distance per
// neighbour kind (the lipids' and the metabolic items' radii are each one
// value in practice, CollisionDistCache recomputes it when they are not).
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS, 4) k_relax_metab_lean(ScParams P, RelaxMArgs A) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;   // list position (count-ordered)
    if (g >= *A.nActivePtr) return;
    const int i = A.L.perm[g];
    if (i < 0) return;
    if (BATCH) rep_apply<BATCH>(P, A.minfo[i].w);
    const float4 v4 = A.mvelIn[i];
    const bool act = P.mAllActive ? i < (int)A.cellStartM[P.cells] : (A.minfo[i].z & SC_ACTIVE) != 0;
    if (!act) {
        A.mvelOut[i] = v4;
        return;
    }
    const int c = A.L.cnt[g];
    if (c > min(SC_LIST_M, P.listLimit)) return;
    const float4 p4 = A.mpos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
    const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
    const sc_f3 ppv = pp + pv;
    sc_f3 dV = sc_zero3();
    float w = 0.0f;
    CollisionDistCache cm, cp;
    const uint32_t *pairs = reinterpret_cast<const uint32_t *>(A.pool) + A.warpOff[g >> 5] + (g & 31);
    uint32_t E[SC_METAB_GROUP];
#pragma unroll
    for (int q = 0; q < SC_METAB_GROUP; q++) E[q] = q < c ? __ldcs(pairs + (size_t)q * 32) : 0u;
    for (int k0 = 0; k0 < c; k0 += SC_METAB_GROUP) {
        float4 t4[SC_METAB_GROUP], tv[SC_METAB_GROUP];
        uint32_t En[SC_METAB_GROUP];
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) {
            const bool on = k0 + q < c;
            const bool fromP = (E[q] & SC_M_FROM_P) != 0;
            const int j = (int)(E[q] & SC_M_INDEX);
            t4[q] = on ? (fromP ? A.ppos : A.mpos)[j] : make_float4(0, 0, 0, 0);
            tv[q] = on ? (fromP ? A.pvel : A.mvelIn)[j] : make_float4(0, 0, 0, 0);
        }
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) {
            const int k = k0 + SC_METAB_GROUP + q;
            En[q] = k < c ? __ldcs(pairs + (size_t)k * 32) : 0u;
        }
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) {
            if (k0 + q < c) {
                const bool fromP = (E[q] & SC_M_FROM_P) != 0;
                const float cd = fromP ? cp.get(p4.w, t4[q].w) : cm.get(p4.w, t4[q].w);
                metab_pair(IM, pp, ppv, t4[q], tv[q], cd, fromP, dV, w);
            }
            E[q] = En[q];
        }
    }
    st3(A.mvelOut, i, pv + dV / fmaxf(w, 1.0f), v4.w);
}

// An item whose list overflowed: the reference's loops over the 27 cells.
template <bool BATCH>
__device__ __forceinline__ void relax_metab_scan_item(const ScParams &P0, const RelaxMArgs &A, int i) {
    if (i < 0) return;
    const int4 mi = A.minfo[i];
    if (!(mi.z & SC_ACTIVE)) return;
    ScParams P = P0;
    rep_apply<BATCH>(P, mi.w);
    float4 v4 = A.mvelIn[i];
    float4 p4 = A.mpos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
    const float prad = p4.w;
    const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
    const sc_f3 ppv = pp + pv;
    sc_f3 dV = sc_zero3();
    float w = 0.0f;
    CollisionDistCache cm, cp;
    const float lim = P.maxInt;
    cells27(P, pp, reach(P, pp, lim, SC_BINNED_M | SC_BINNED_P), [&](uint32_t key) {
        for (uint32_t j = A.cellStartM[key], e = A.cellStartM[key + 1]; j < e; j++) {
            if ((int)j == i) continue;
            if (!active_m(P, A.minfo, (int)j)) continue;
            float4 t4 = A.mpos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) continue;
            if (cm.collides(prad, t4.w, delta))
                metab_pair(IM, pp, ppv, t4, A.mvelIn[j], cm.get(prad, t4.w), false, dV, w);
        }
        for (uint32_t j = A.cellStartP[key], e = A.cellStartP[key + 1]; j < e; j++) {
            if (!active_lipid(P, A.pinfo, (int)j)) continue;
            float4 t4 = A.ppos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) continue;
            if (cp.collides(prad, t4.w, delta))
                metab_pair(IM, pp, ppv, t4, A.pvel[j], cp.get(prad, t4.w), true, dV, w);
        }
    });
    st3(A.mvelOut, i, pv + dV / fmaxf(w, 1.0f), v4.w);
}

// Lists of the overflow pool longer than this are walked by a whole warp,
// shorter ones by one thread (both in k_relax_metab_pool): a list that
// overflowed because the main pool had no room for its block fits the list
// capacity, one that outgrew the capacity (a wall pile's) holds hundreds to
// thousands of pairs.  With the list capacity capped (pair_list_limit, the
// tests' way into the overflow paths) the bound is four times the cap, so
// ordinary lists take both walks.
#define SC_POOL_WARP_MIN SC_LIST_M
__device__ __forceinline__ int pool_warp_min(const ScParams &P) {
    return P.listLimit < SC_POOL_WARP_MIN / 4 ? 4 * P.listLimit : SC_POOL_WARP_MIN;
}

// The items whose list overflowed (listed by k_build_m), a thread each,
// grid-stride: an item the overflow pool had no room for scans its
// neighbourhood; one whose region there is short walks it as k_relax_metab
// walks the main pool (the same terms in the same order, SC_METAB_GROUP pairs
// in flight); the long regions are k_relax_metab_pool's.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_relax_metab_overflow(ScParams P, RelaxMArgs A,
                                                                     const int *__restrict__ ovf,
                                                                     const int *__restrict__ ovfCount,
                                                                     const int *__restrict__ ovfN,
                                                                     const long long *__restrict__ ovfOff,
                                                                     const uint4 *__restrict__ ovfPool) {
    const int warpMin = pool_warp_min(P);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *ovfCount; t += gridDim.x * blockDim.x) {
        const int i = ovf[t];
        const long long off = ovfOff ? ovfOff[t] : -1;
        if (off < 0) {
            relax_metab_scan_item<BATCH>(P, A, i);
            continue;
        }
        const int n = ovfN[t];
        if (i < 0 || n > warpMin || !(A.minfo[i].z & SC_ACTIVE)) continue;
        const float4 v4 = A.mvelIn[i], p4 = A.mpos[i];
        const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
        const sc_f3 ppv = sc_make_f3(p4.x, p4.y, p4.z) + pv;
        sc_f3 dV = sc_zero3();
        float w = 0.0f;
        const uint4 *__restrict__ e = ovfPool + off;
        uint4 E[SC_METAB_GROUP];
#pragma unroll
        for (int q = 0; q < SC_METAB_GROUP; q++) E[q] = q < n ? e[q] : make_uint4(0, 0, 0, 0);
        for (int k0 = 0; k0 < n; k0 += SC_METAB_GROUP) {
            float4 tv[SC_METAB_GROUP];
            uint4 En[SC_METAB_GROUP];
#pragma unroll
            for (int q = 0; q < SC_METAB_GROUP; q++)
                tv[q] = k0 + q < n ? metab_pair_vel(A, E[q].x) : make_float4(0, 0, 0, 0);
#pragma unroll
            for (int q = 0; q < SC_METAB_GROUP; q++) {
                const int k = k0 + SC_METAB_GROUP + q;
                En[q] = k < n ? e[k] : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int q = 0; q < SC_METAB_GROUP; q++) {
                if (k0 + q < n) {
                    const float kw = (E[q].x & SC_M_FROM_P) ? 2.0f : 1.0f;
                    const sc_f3 a = sc_make_f3(__uint_as_float(E[q].y), __uint_as_float(E[q].z),
                                               __uint_as_float(E[q].w));
                    w += kw;
                    dV += (a + sc_make_f3(tv[q].x, tv[q].y, tv[q].z) - ppv) * 0.9f * kw;
                }
                E[q] = En[q];
            }
        }
        st3(A.mvelOut, i, pv + dV / fmaxf(w, 1.0f), v4.w);
    }
}

// The overflowed items whose list is kept whole in the overflow pool
// (k_build_m_ovf) and is longer than pool_warp_min, a warp each, warp-stride
// over the items so the long lists of a wall pile spread over the device:
// the lanes load 32 entries and the neighbours' velocities at once and each
// forms its pair's term and weight; lanes 0-2 add the terms' components and
// lane 3 the weights in list order from shared memory -- the sums a thread
// walking the list forms, at one gather latency per 32 pairs.
__global__ void __launch_bounds__(SC_THREADS) k_relax_metab_pool(ScParams P, RelaxMArgs A, const int *__restrict__ ovf,
                                                                 const int *__restrict__ ovfCount,
                                                                 const int *__restrict__ ovfN,
                                                                 const long long *__restrict__ ovfOff,
                                                                 const uint4 *__restrict__ ovfPool) {
    __shared__ float sTerm[SC_THREADS / 32][32][5];   // x, y, z, weight (odd row length: no bank conflicts)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nOvf = *ovfCount;
    const int warpMin = pool_warp_min(P);
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nOvf; t += (gridDim.x * blockDim.x) >> 5) {
        const int i = ovf[t], n = ovfN[t];
        const long long off = ovfOff[t];
        if (off < 0 || i < 0 || n <= warpMin || !(A.minfo[i].z & SC_ACTIVE)) continue;   // warp-uniform
        const float4 v4 = A.mvelIn[i], p4 = A.mpos[i];
        const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
        const sc_f3 ppv = sc_make_f3(p4.x, p4.y, p4.z) + pv;
        const uint4 *__restrict__ e = ovfPool + off;
        float acc = 0.0f;   // lanes 0-2: dV's components; lane 3: the weight
        for (int b = 0; b < n; b += 32) {
            float term[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (b + lane < n) {
                const uint4 E = e[b + lane];
                const float4 tv = metab_pair_vel(A, E.x);
                const float kw = (E.x & SC_M_FROM_P) ? 2.0f : 1.0f;
                const sc_f3 a = sc_make_f3(__uint_as_float(E.y), __uint_as_float(E.z), __uint_as_float(E.w));
                const sc_f3 d = (a + sc_make_f3(tv.x, tv.y, tv.z) - ppv) * 0.9f * kw;
                term[0] = d.x;
                term[1] = d.y;
                term[2] = d.z;
                term[3] = kw;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) sTerm[wid][lane][k] = term[k];
            __syncwarp();
            if (lane < 4) {
                const int m = min(32, n - b);
                for (int u = 0; u < m; u++) acc += sTerm[wid][u][lane];
            }
            __syncwarp();
        }
        const float dy = __shfl_sync(0xffffffffu, acc, 1), dz = __shfl_sync(0xffffffffu, acc, 2),
                    w = __shfl_sync(0xffffffffu, acc, 3);
        if (lane == 0) st3(A.mvelOut, i, pv + sc_make_f3(acc, dy, dz) / fmaxf(w, 1.0f), v4.w);
    }
}

// ---- the same sweep on column-segment tiles (sc_tile.cuh) ---------------------
// Shared-memory header of a tile block; the tile arrays follow it.
struct TileMHeader {
    uint64_t bar;
    int nItems;
    int runBase[SC_TILE_NITEMCOL], runStart[SC_TILE_NITEMCOL + 1];
    TileRanges RM, RP;
};
#define SC_TILE_HDR_BYTES ((sizeof(TileMHeader) + 127) / 128 * 128)

// The block's geometry, both range tables and its item runs (the inner
// columns over [z0, z1)); ends with a block barrier.
__device__ __forceinline__ void tile_m_setup(const ScParams &P, const TileGeom &G, const uint32_t *__restrict__ cellStartM,
                                             const uint32_t *__restrict__ cellStartP, TileMHeader &H) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tile_ranges(P, G, cellStartM, 0, P.tileCapM, H.RM);
    if (warp == 1) tile_ranges(P, G, cellStartP, P.tileCapM, P.tileCapP, H.RP);
    if (warp == 2) {
        int b = 0, l = 0;
        if (lane < SC_TILE_NITEMCOL) {
            const int gx = G.x0 + lane / SC_TILE_TY, gy = G.y0 + lane % SC_TILE_TY;
            if (gx < G.n && gy < G.n) {
                const uint32_t k0 = cell_key(P, (uint32_t)gx, (uint32_t)gy, 0);
                b = (int)cellStartM[k0 + (uint32_t)G.z0];
                l = (int)cellStartM[k0 + (uint32_t)G.z1] - b;
            }
        }
        int x = l;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < SC_TILE_NITEMCOL) {
            H.runBase[lane] = b;
            H.runStart[lane] = x - l;
        }
        if (lane == SC_TILE_NITEMCOL - 1) {
            H.runStart[SC_TILE_NITEMCOL] = x;
            H.nItems = x;
        }
    }
    __syncthreads();
}
// Slot of the block's t-th item.
__device__ __forceinline__ int tile_item(const TileMHeader &H, int t) {
    int q = 0;
#pragma unroll
    for (int k = 1; k < SC_TILE_NITEMCOL; k++) q += t >= H.runStart[k];
    return H.runBase[q] + (t - H.runStart[q]);
}

// Packed 16-bit list entries: 8 consecutive entries of an item share one
// 16-byte chunk, chunks warp-tiled (chunk q of item i at
// ((i/32) * K/8 + q) * 32 + i%32), so one load brings 8 entries.
__host__ __device__ __forceinline__ size_t sc_list16_at(int K, int i, int k) {
    return (((size_t)(i >> 5) * (size_t)(K / 8) + (size_t)(k >> 3)) * 32 + (size_t)(i & 31)) * 8 + (size_t)(k & 7);
}

// M list on tiles: entries are 16-bit tile offsets (metabolic slots first,
// then particle slots), in the reference's visiting order, packed.  An item whose
// neighbourhood leaves the tile, or whose list would overflow, is listed in
// `ovf` for the scanning kernel.
__global__ void __launch_bounds__(SC_THREADS) k_build_m_tile(ScParams P, const uint32_t *__restrict__ cellStartM,
                                                             const uint32_t *__restrict__ cellStartP,
                                                             const float4 *__restrict__ mpos, const int4 *__restrict__ minfo,
                                                             const float4 *__restrict__ ppos_, const int4 *__restrict__ pinfo,
                                                             uint16_t *__restrict__ list, int *__restrict__ cnt,
                                                             int *__restrict__ ovf, int *__restrict__ ovfCount) {
    extern __shared__ __align__(128) unsigned char smraw[];
    TileMHeader &H = *reinterpret_cast<TileMHeader *>(smraw);
    const int cap = P.tileCapM + P.tileCapP;
    float4 *spos = reinterpret_cast<float4 *>(smraw + SC_TILE_HDR_BYTES);
    uint8_t *sok = reinterpret_cast<uint8_t *>(spos + cap);
    TileGeom G;
    G.init(P, blockIdx.x);
    tile_m_setup(P, G, cellStartM, cellStartP, H);
    for (int r = 0; r < SC_TILE_NRANGE; r++) {
        for (int k = threadIdx.x; k < H.RM.len[r]; k += blockDim.x) {
            const int j = H.RM.base[r] + k, o = H.RM.off[r] + k;
            spos[o] = mpos[j];
            sok[o] = (minfo[j].z & SC_ACTIVE) ? 1 : 0;
        }
        for (int k = threadIdx.x; k < H.RP.len[r]; k += blockDim.x) {
            const int j = H.RP.base[r] + k, o = H.RP.off[r] + k;
            const int4 tin = pinfo[j];
            spos[o] = ppos_[j];
            sok[o] = ((tin.z & SC_ACTIVE) && tin.y == SC_PARTICLE_TYPE_LIPID) ? 1 : 0;
        }
    }
    __syncthreads();
    const int bits = P.bits;
    const uint32_t zmask = (1u << bits) - 1u;
    for (int t = threadIdx.x; t < H.nItems; t += blockDim.x) {
        const int i = tile_item(H, t);
        if (!(minfo[i].z & SC_ACTIVE)) {
            cnt[i] = 0;
            continue;
        }
        float4 p4 = mpos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
        const float prad = p4.w, lim = P.maxInt;
        CollisionDistCache cm, cp;
        int c = 0;
        bool miss = false;
        const int climit = min(SC_LIST_M, P.listLimit);
        cells27(P, pp, reach(P, pp, lim, SC_BINNED_M | SC_BINNED_P), [&](uint32_t key) {
            if (miss) return;
            const int r = G.range_of((int)(key >> (2 * bits)), (int)((key >> bits) & zmask), (int)(key & zmask));
            const int am = (int)cellStartM[key], em = (int)cellStartM[key + 1];
            const int ap = (int)cellStartP[key], ep = (int)cellStartP[key + 1];
            // a non-empty cell outside the tile, or clipped by its capacity
            if ((em > am && (r < 0 || am - H.RM.base[r] + (em - am) > H.RM.len[r])) ||
                (ep > ap && (r < 0 || ap - H.RP.base[r] + (ep - ap) > H.RP.len[r]))) {
                miss = true;
                return;
            }
            for (int j = am; j < em; j++) {
                const int o = H.RM.off[r] + (j - H.RM.base[r]);
                if (j == i || !sok[o]) continue;
                float4 t4 = spos[o];
                sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
                if (outside_cube(delta, lim)) continue;
                if (cm.collides(prad, t4.w, delta)) {
                    if (c < climit) list[sc_list16_at(SC_LIST_M, i, c)] = (uint16_t)o;
                    c++;
                }
            }
            for (int j = ap; j < ep; j++) {
                const int o = H.RP.off[r] + (j - H.RP.base[r]);
                if (!sok[o]) continue;
                float4 t4 = spos[o];
                sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
                if (outside_cube(delta, lim)) continue;
                if (cp.collides(prad, t4.w, delta)) {
                    if (c < climit) list[sc_list16_at(SC_LIST_M, i, c)] = (uint16_t)o;
                    c++;
                }
            }
        });
        if (miss || c > climit) {
            cnt[i] = INT_MAX;
            ovf[atomicAdd(ovfCount, 1)] = i;
        } else {
            cnt[i] = c;
        }
    }
}

// relaxMetabolicParticles on tiles: the block bulk-copies the positions and
// velocities of its tile, then walks each item's list in shared memory.
__global__ void __launch_bounds__(SC_THREADS) k_relax_metab_tile(ScParams P, RelaxMArgs A,
                                                                 const uint16_t *__restrict__ list,
                                                                 int *__restrict__ errorFlag) {
    extern __shared__ __align__(128) unsigned char smraw[];
    TileMHeader &H = *reinterpret_cast<TileMHeader *>(smraw);
    const int capM = P.tileCapM, cap = P.tileCapM + P.tileCapP;
    float4 *spos = reinterpret_cast<float4 *>(smraw + SC_TILE_HDR_BYTES);
    float4 *svel = spos + cap;
    // after an expired wait anywhere, the remaining blocks do nothing
    if (*(volatile int *)errorFlag == SC_DERR_TILE_TIMEOUT) return;
    TileGeom G;
    G.init(P, blockIdx.x);
    if (threadIdx.x == 0) mbar_init(&H.bar);
    tile_m_setup(P, G, A.cellStartM, A.cellStartP, H);
    if (threadIdx.x < 32) {  // warp 0 issues the bulk copies, a lane per range
        const int lane = threadIdx.x;
        uint32_t bytes = 0;
        for (int r = lane; r < SC_TILE_NRANGE; r += 32)
            bytes += 32u * (uint32_t)(max(H.RM.len[r], 0) + max(H.RP.len[r], 0));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
        if (lane == 0) mbar_expect_tx(&H.bar, bytes);
        __syncwarp();
        for (int r = lane; r < SC_TILE_NRANGE; r += 32) {
            if (H.RM.len[r] > 0) {
                const uint32_t nb = (uint32_t)H.RM.len[r] * 16u;
                bulk_copy(spos + H.RM.off[r], A.mpos + H.RM.base[r], nb, &H.bar);
                bulk_copy(svel + H.RM.off[r], A.mvelIn + H.RM.base[r], nb, &H.bar);
            }
            if (H.RP.len[r] > 0) {
                const uint32_t nb = (uint32_t)H.RP.len[r] * 16u;
                bulk_copy(spos + H.RP.off[r], A.ppos + H.RP.base[r], nb, &H.bar);
                bulk_copy(svel + H.RP.off[r], A.pvel + H.RP.base[r], nb, &H.bar);
            }
        }
    }
    // the thread's first item is loaded while the tile is in flight
    const int climit = min(SC_LIST_M, P.listLimit);
    int t = threadIdx.x;
    int i = t < H.nItems ? tile_item(H, t) : -1;
    int4 in = i >= 0 ? A.minfo[i] : make_int4(0, 0, 0, 0);
    int c = i >= 0 ? A.L.cnt[i] : 0;
    float4 v4 = i >= 0 ? A.mvelIn[i] : make_float4(0, 0, 0, 0);
    float4 p4 = i >= 0 ? A.mpos[i] : make_float4(0, 0, 0, 0);
    if (!mbar_wait_bounded(&H.bar, 1ll << 31)) {
        if (threadIdx.x == 0) atomicCAS(errorFlag, 0, SC_DERR_TILE_TIMEOUT);
        mbar_wait_bounded(&H.bar, 1ll << 31);   // let the copies in flight land before the block exits
        return;
    }
    for (; t < H.nItems; t += blockDim.x) {
        if (t != (int)threadIdx.x) {
            i = tile_item(H, t);
            in = A.minfo[i];
            c = A.L.cnt[i];
            v4 = A.mvelIn[i];
            p4 = A.mpos[i];
        }
        if (!(in.z & SC_ACTIVE)) {
            A.mvelOut[i] = v4;
            continue;
        }
        if (c > climit) continue;
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_M | SC_BINNED_P);
        const float prad = p4.w;
        const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
        const sc_f3 ppv = pp + pv;
        sc_f3 dV = sc_zero3();
        float w = 0.0f;
        CollisionDistCache cm, cp;
        // 8 entries per load; the next chunk is loaded while this one is walked
        const uint4 *__restrict__ chunks = reinterpret_cast<const uint4 *>(list) +
                                           (size_t)(i >> 5) * (SC_LIST_M / 8) * 32 + (i & 31);
        uint4 cur = c > 0 ? chunks[0] : make_uint4(0, 0, 0, 0);
        for (int q = 0; 8 * q < c; q++) {
            const uint4 nxt = 8 * (q + 1) < c ? chunks[(size_t)(q + 1) * 32] : make_uint4(0, 0, 0, 0);
            const uint32_t words[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
                if (8 * q + kk >= c) break;
                const uint32_t e = (words[kk >> 1] >> (16 * (kk & 1))) & 0xffffu;
                const float4 t4 = spos[e], tv = svel[e];
                const bool fromP = (int)e >= capM;
                const float cd = fromP ? cp.get(prad, t4.w) : cm.get(prad, t4.w);
                metab_pair(IM, pp, ppv, t4, tv, cd, fromP, dV, w);
            }
            cur = nxt;
        }
        st3(A.mvelOut, i, pv + dV / fmaxf(w, 1.0f), v4.w);
    }
}

// Velocities of the slots past the binned items (inactive since the sort).
__global__ void __launch_bounds__(SC_THREADS) k_copy_tail(const uint32_t *__restrict__ binnedEnd,
                                                          const int *__restrict__ nActivePtr,
                                                          const float4 *__restrict__ in, float4 *__restrict__ out) {
    const int n = *nActivePtr;
    for (int i = (int)*binnedEnd + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = in[i];
}

// ---- metabolites.cuh:266-350 relaxMetabolicParticlePartners ----------------
// Only lipids change, and only their own velocity, which no other thread of
// this kernel reads: updated in place.  List: the colliding metabolic items.
__device__ __forceinline__ void build_lm_item(const ScParams &P, const uint32_t *__restrict__ cellStartM, int i,
                                              const float4 *__restrict__ ppos_, const float4 *__restrict__ mpos,
                                              const int4 *__restrict__ minfo, uint32_t *list, int &c) {
    float4 p4 = ppos_[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M);
    const float prad = p4.w, lim = P.maxInt;
    CollisionDistCache cc;
    scan27(P, cellStartM, pp, reach(P, pp, lim, SC_BINNED_M), [&](int j) {
        if (!active_m(P, minfo, j)) return;
        float4 t4 = mpos[j];
        sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
        if (outside_cube(delta, lim)) return;
        if (cc.collides(prad, t4.w, delta)) {
            if (c < min(SC_LIST_LM, P.listLimit)) list[sc_list_at(SC_LIST_LM, i, c)] = (uint32_t)j;
            c++;
        }
    });
}

// LM pairs with their frozen geometry, as the M pairs: per pair
// A = tpos - normalize(tpos - pos) * collisionDistance
// (metabolites.cuh:320-332), the first float3 the reference's velocity term
// evaluates, in a pool region of the list position's warp (pool_take),
// 16 bytes {neighbour, A.x, A.y, A.z} per entry.  An overflowed lipid
// (cnt INT_MAX) is left to the scan of k_relax_partners.
// The active lipids, compacted (warp-aggregated appends: the order of the
// lists does not matter, each lipid's own list keeps the scan's order), so
// the LM build's warps hold only lipids.
__global__ void __launch_bounds__(SC_THREADS) k_lipid_select(const int *__restrict__ nActivePtr,
                                                             const int4 *__restrict__ pinfo, int *__restrict__ work,
                                                             int *__restrict__ workCount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool lip = false;
    if (i < *nActivePtr) {
        const int4 in = pinfo[i];
        lip = (in.z & SC_ACTIVE) && in.y == SC_PARTICLE_TYPE_LIPID;
    }
    const unsigned m = __ballot_sync(0xffffffffu, lip);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(workCount, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (lip) work[base + __popc(m & ((1u << lane) - 1u))] = i;
}

template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_lm(ScParams P0, const uint32_t *__restrict__ cellStartM,
                                                         const int *__restrict__ lipids,
                                                         const int *__restrict__ lipidCount,
                                                         const int4 *__restrict__ pinfo,
                                                         const float4 *__restrict__ ppos_,
                                                         const float4 *__restrict__ mpos, const int4 *__restrict__ minfo,
                                                         uint4 *__restrict__ pool, long long poolCap,
                                                         unsigned long long *__restrict__ poolUsed,
                                                         long long *__restrict__ warpOff,
                                                         uint32_t *scratch, int *__restrict__ cnt,
                                                         int *__restrict__ perm, int cap) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < *lipidCount;
    int c = 0;
    if (valid) {
        ScParams P = P0;
        rep_apply<BATCH>(P, pinfo[lipids[t]].w);
        build_lm_item(P, cellStartM, lipids[t], ppos_, mpos, minfo, scratch, c);
    }
    const PoolSlot<uint4> S = pool_take<SC_LIST_LM>(P0, valid, c, pool, poolCap, poolUsed, warpOff, cnt, perm, cap,
                                                    nullptr, nullptr, lipids);
    if (S.n == 0) return;
    ScParams P = P0;
    rep_apply<BATCH>(P, pinfo[S.i].w);
    const float4 p4 = ppos_[S.i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M);
    const float prad = p4.w;
    CollisionDistCache cc;
    for (int k = 0; k < S.n; k++) {
        const uint32_t j = scratch[sc_list_at(SC_LIST_LM, S.i, k)];
        const float4 t4 = mpos[j];
        const sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
        const sc_f3 nd = normalize(tpos - pp);
        const sc_f3 a = tpos - nd * cc.get(prad, t4.w);
        S.out[(size_t)k * 32] = make_uint4(j, __float_as_uint(a.x), __float_as_uint(a.y), __float_as_uint(a.z));
    }
}

// metabolites.cuh:267-340 for one lipid: each listed metabolic neighbour
// adds its precomputed geometry and current velocity with weight 2, in list
// order; the pairs are taken four at a time (entries, then velocities, all
// in flight together).  An overflowed lipid scans its neighbourhood.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_relax_partners(
    ScParams P, const uint32_t *__restrict__ cellStartM, const int *__restrict__ nActivePtr,
    const float4 *__restrict__ ppos_, const int4 *__restrict__ pinfo, float4 *__restrict__ pvel_,
    PairList<SC_LIST_LM> L, const uint4 *__restrict__ pool, const long long *__restrict__ warpOff,
    const float4 *__restrict__ mpos, const int4 *__restrict__ minfo, const float4 *__restrict__ mvel) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;   // list position (count-ordered)
    if (g >= *nActivePtr) return;
    const int i = L.perm[g];
    if (i < 0) return;
    int4 in = pinfo[i];
    if (!(in.z & SC_ACTIVE) || in.y != SC_PARTICLE_TYPE_LIPID) return;
    rep_apply<BATCH>(P, in.w);
    float4 p4 = ppos_[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const float prad = p4.w;
    float4 v4 = pvel_[i];
    const sc_f3 pv = sc_make_f3(v4.x, v4.y, v4.z);
    sc_f3 dV = sc_zero3();
    float w = 0.0f;
    const int c = L.cnt[g];
    if (c <= min(SC_LIST_LM, P.listLimit)) {
        const uint4 *pairs = pool + warpOff[g >> 5] + (g & 31);
        for (int k0 = 0; k0 < c; k0 += 4) {
            uint4 E[4];
            float4 tv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) E[q] = k0 + q < c ? __ldcs(pairs + (size_t)(k0 + q) * 32) : make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int q = 0; q < 4; q++) tv[q] = k0 + q < c ? mvel[E[q].x] : make_float4(0, 0, 0, 0);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (k0 + q < c) {
                    const sc_f3 a = sc_make_f3(__uint_as_float(E[q].y), __uint_as_float(E[q].z), __uint_as_float(E[q].w));
                    w += 2.0f;
                    dV += (a + sc_make_f3(tv[q].x, tv[q].y, tv[q].z) - (pp + pv)) * 0.9f * 2.0f;
                }
            }
        }
    } else {
        const Imager IM(P, pp, SC_BINNED_M);
        CollisionDistCache cc;
        const float lim = P.maxInt;
        scan27(P, cellStartM, pp, reach(P, pp, lim, SC_BINNED_M), [&](int j) {
            if (!active_m(P, minfo, j)) return;
            float4 t4 = mpos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) return;
            if (cc.collides(prad, t4.w, delta)) {
                const float cd = cc.cd;
                sc_f3 tpos = IM(sc_make_f3(t4.x, t4.y, t4.z));
                sc_f3 nd = normalize(tpos - pp);
                w += 2.0f;
                dV += (tpos - nd * cd + ld3(mvel, j) - (pp + pv)) * 0.9f * 2.0f;
            }
        });
    }
    st3(pvel_, i, pv + dV / fmaxf(w, 1.0f), v4.w);
}

// Alignment tests of complexify / transitionInteractions (interactions.cuh:319-324, 438-443).
__device__ __forceinline__ void alignment(bool ord, sc_f4 prot, sc_f4 trot, sc_f3 up, sc_f3 tup, sc_f3 delta,
                                          const sc_rule &r, float *oa, float *rpa) {
    sc_f4 ro = rule_ori(r);
    sc_f3 rp = rule_pos(r);
    *oa = ord ? dot(sc_rotate(up, ro), tup) : dot(sc_rotate(tup, ro), up);
    *rpa = ord ? dot(sc_rotate(rp, prot), delta) / sc_normsq3(delta)
               : dot(sc_rotate(rp, trot), -delta) / sc_normsq3(delta);
}
__device__ __forceinline__ bool states_match(bool ord, int ps, int ts, const sc_rule &r) {
    int fs = r.first_partner_state, ss = r.second_partner_state;
    return ord ? ((fs < 0 || fs == ps) && (ss < 0 || ss == ts)) : ((ss < 0 || ss == ps) && (fs < 0 || fs == ts));
}
__device__ __forceinline__ bool group_active_in(const int *__restrict__ b, int nbv, int group) {
    for (int k = 0; k < min(nbv, SC_MAX_ACTIVE_INTERACTIONS); k++)
        if (b[3 * k + 1] == group) return true;
    return false;
}

// ---- interactions.cuh:216-346 complexify --------------------------------------
// New interactions are appended at slots [nb, nb') of the item's own list,
// which no neighbour reads (they read [0, nb)); nb' goes to the next buffer.
// The items complexify can act on, collected before the scan so the scan's
// warps hold only such items (they are a small, scattered part of the
// particles: left in place, almost every warp would carry one or two
// scanning lanes).  No rule of an item's type can add a bond when each is
// transition-only or its group is already active on the item (bonds are
// only added by the scan, so a blocked rule stays blocked); such an item's
// bond count is passed through here.
__global__ void __launch_bounds__(SC_THREADS) k_complexify_select(ScParams P, const int *__restrict__ nActivePtr,
                                                                  const int4 *__restrict__ info,
                                                                  const int *__restrict__ nbIn,
                                                                  int *__restrict__ nbOut,
                                                                  const int *__restrict__ bonds,
                                                                  int *__restrict__ work, int *__restrict__ workCount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool open = false;
    if (i < *nActivePtr) {
        const int4 in = info[i];
        const int pnb = nbIn[i];
        int cs = 0, ce = 0;
        if ((in.z & SC_ACTIVE) && in.y >= 0 && 2 * in.y + 1 < P.nPidx) {
            cs = P.pidx[2 * in.y];
            ce = P.pidx[2 * in.y + 1];
        }
        for (int k = cs; k < ce && !open && pnb < SC_MAX_ACTIVE_INTERACTIONS; k++) {
            const sc_rule &pii = P.prules[k];
            open = !pii.only_via_transition &&
                   !(pii.group >= 0 && group_active_in(bonds + (size_t)i * 24, pnb, pii.group));
        }
        if (!open) nbOut[i] = pnb;
    }
    // warp-aggregated append (order within the list is free: items do not read what others add)
    const unsigned m = __ballot_sync(0xffffffffu, open);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(workCount, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (open) work[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// The binding draw of a rule with a probability (an extension; the
// reference's rules carry none and always pass).
__device__ __forceinline__ bool bind_draw(const ScParams &P, const sc_rule &r, int pid, int tid, int step) {
    return !r.use_probability || sc_bind_uniform(P.seed, r.id, pid, tid, step) < r.probability;
}

template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_complexify(
    ScParams P, const uint32_t *__restrict__ cellStart, const int *__restrict__ work, const int *__restrict__ workCount,
    const float4 *__restrict__ pos, const float4 *__restrict__ rot, const int4 *__restrict__ info,
    const int *__restrict__ state, const int *__restrict__ nbIn, int *__restrict__ nbOut, int *bonds,
    const int *__restrict__ stepPtr, int prep) {
  const int step = prep ? -1 : *stepPtr;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *workCount; t += gridDim.x * blockDim.x) {
    const int i = work[t];
    int4 in = info[i];
    rep_apply<BATCH>(P, in.w);
    int pnb = nbIn[i];
    const int cs = P.pidx[2 * in.y], ce = P.pidx[2 * in.y + 1];
    float4 p4 = pos[i];
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, ppos, SC_BINNED_P);
    const sc_f4 prot = ld4(rot, i);
    const int pid = in.x, ptype = in.y, pstate = state[i];
    const sc_f3 up = sc_rotate(sc_up(), prot);
    int *pb = bonds + (size_t)i * 24;
    const int nb0 = pnb;
    const float lim = P.maxInt;
    scan27(P, cellStart, ppos, reach(P, ppos, lim, SC_BINNED_P), [&](int j) {
        if (j == i) return;
        float4 t4 = pos[j];
        sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - ppos;
        if (outside_cube(delta, lim)) return;
        int4 tin = info[j];
        if (!(tin.z & SC_ACTIVE)) return;
        sc_f4 trot = ld4(rot, j);
        sc_f3 tup = sc_rotate(sc_up(), trot);
        const int ttype = tin.y;
        bool ord = p_order(ptype, pid, ttype, tin.x);
        for (int k = cs; k < ce; k++) {
            if (pnb >= SC_MAX_ACTIVE_INTERACTIONS) continue;
            const sc_rule &pii = P.prules[k];
            if (!((ptype == pii.first_partner_type && ttype == pii.second_partner_type) ||
                  (ptype == pii.second_partner_type && ttype == pii.first_partner_type)) ||
                pii.only_via_transition)
                continue;
            if (pii.group >= 0 && (group_active_in(pb, pnb, pii.group) ||
                                   group_active_in(bonds + (size_t)j * 24, nbIn[j], pii.group)))
                continue;
            float oa, rpa;
            alignment(ord, prot, trot, up, tup, delta, pii, &oa, &rpa);
            if (oa > pii.orientation_alignment_threshold &&
                fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold) &&
                states_match(ord, pstate, state[j], pii) && bind_draw(P, pii, pid, tin.x, step)) {
                pb[3 * pnb] = pii.id;
                pb[3 * pnb + 1] = pii.group;
                pb[3 * pnb + 2] = tin.x;
                pnb++;
            }
        }
    });
    (void)nb0;
    nbOut[i] = pnb;
  }
}

// ---- complexify by deterministic pair claim (sc_config.pair_claim) ----------
// The reference's scan appends a bond on the scanning item's side only, so
// two items can both bond a third that keeps just one of them (the TODO at
// interactions.cuh:297).  Here a step forms rule bonds in two kernels:
//   offer: every open item i that has a free bond slot visits its
//          neighbours as complexify does and, for each neighbour j that some
//          rule would bond it to, lowers claim[j] to the 64-bit key
//          (bits of |delta|^2, i) with atomicMin;
//   bind:  i and j bond when claim[i] names j and claim[j] names i.  Both
//          sides take the first rule that passes for the pair as seen from
//          the lower slot, so the two records always agree.
// At most one rule bond forms per item per step.  Keys and slots are fixed by
// the sort, so the result does not depend on thread scheduling.
struct ClaimItem {
    sc_f3 pos, up;
    sc_f4 rot;
    int id, type, state, nb, cs, ce;
    const int *b;
};
__device__ __forceinline__ ClaimItem claim_item(const ScParams &P, const float4 *__restrict__ pos,
                                                const float4 *__restrict__ rot, const int4 *__restrict__ info,
                                                const int *__restrict__ state, const int *__restrict__ nbIn,
                                                const int *bonds, int i) {
    ClaimItem a;
    const float4 p4 = pos[i];
    a.pos = sc_make_f3(p4.x, p4.y, p4.z);
    a.rot = ld4(rot, i);
    a.up = sc_rotate(sc_up(), a.rot);
    const int4 in = info[i];
    a.id = in.x;
    a.type = in.y;
    a.state = state[i];
    a.nb = nbIn[i];
    a.b = bonds + (size_t)i * 24;
    a.cs = a.ce = 0;
    if (in.y >= 0 && 2 * in.y + 1 < P.nPidx) {
        a.cs = P.pidx[2 * in.y];
        a.ce = P.pidx[2 * in.y + 1];
    }
    return a;
}
// The partner-mapped index of the first rule of a's type that would bond a
// to b (delta = b's position seen from a, minus a's), or -1.
__device__ __forceinline__ int claim_rule(const ScParams &P, const ClaimItem &a, const ClaimItem &b, sc_f3 delta,
                                          int step) {
    if (a.nb >= SC_MAX_ACTIVE_INTERACTIONS) return -1;
    const bool ord = p_order(a.type, a.id, b.type, b.id);
    for (int k = a.cs; k < a.ce; k++) {
        const sc_rule &pii = P.prules[k];
        if (!((a.type == pii.first_partner_type && b.type == pii.second_partner_type) ||
              (a.type == pii.second_partner_type && b.type == pii.first_partner_type)) ||
            pii.only_via_transition)
            continue;
        if (pii.group >= 0 && (group_active_in(a.b, a.nb, pii.group) || group_active_in(b.b, b.nb, pii.group)))
            continue;
        float oa, rpa;
        alignment(ord, a.rot, b.rot, a.up, b.up, delta, pii, &oa, &rpa);
        if (oa > pii.orientation_alignment_threshold &&
            fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold) &&
            states_match(ord, a.state, b.state, pii) && bind_draw(P, pii, a.id, b.id, step))
            return k;
    }
    return -1;
}
__device__ __forceinline__ unsigned long long claim_key(sc_f3 delta, int i) {
    return ((unsigned long long)sc_f2u(sc_normsq3(delta)) << 32) | (unsigned)i;
}

template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS, 3) k_claim_offer(
    ScParams P, const uint32_t *__restrict__ cellStart, const int *__restrict__ work, const int *__restrict__ workCount,
    const float4 *__restrict__ pos, const float4 *__restrict__ rot, const int4 *__restrict__ info,
    const int *__restrict__ state, const int *__restrict__ nbIn, const int *__restrict__ bonds,
    const int *__restrict__ stepPtr, int prep, unsigned long long *claim) {
  const int step = prep ? -1 : *stepPtr;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *workCount; t += gridDim.x * blockDim.x) {
    const int i = work[t];
    rep_apply<BATCH>(P, info[i].w);
    const ClaimItem a = claim_item(P, pos, rot, info, state, nbIn, bonds, i);
    if (a.nb >= SC_MAX_ACTIVE_INTERACTIONS) continue;
    const Imager IM(P, a.pos, SC_BINNED_P);
    const float lim = P.maxInt;
    scan27(P, cellStart, a.pos, reach(P, a.pos, lim, SC_BINNED_P), [&](int j) {
        if (j == i) return;
        const float4 t4 = pos[j];
        const sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - a.pos;
        if (outside_cube(delta, lim)) return;
        if (!(info[j].z & SC_ACTIVE)) return;
        const ClaimItem b = claim_item(P, pos, rot, info, state, nbIn, bonds, j);
        if (claim_rule(P, a, b, delta, step) >= 0) atomicMin(&claim[j], claim_key(delta, i));
    });
  }
}

template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_claim_bind(
    ScParams P, const int *__restrict__ work, const int *__restrict__ workCount, const float4 *__restrict__ pos,
    const float4 *__restrict__ rot, const int4 *__restrict__ info, const int *__restrict__ state,
    const int *__restrict__ nbIn, int *__restrict__ nbOut, int *bonds, const int *__restrict__ stepPtr, int prep,
    const unsigned long long *__restrict__ claim) {
  const int step = prep ? -1 : *stepPtr;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *workCount; t += gridDim.x * blockDim.x) {
    const int i = work[t];
    int pnb = nbIn[i];
    const unsigned long long key = claim[i];
    const int j = (int)(unsigned)(key & 0xffffffffull);
    if (key != ~0ull && (int)(unsigned)(claim[j] & 0xffffffffull) == i) {
        const int lo = min(i, j), hi = max(i, j);
        rep_apply<BATCH>(P, info[lo].w);
        const ClaimItem a = claim_item(P, pos, rot, info, state, nbIn, bonds, lo);
        const ClaimItem b = claim_item(P, pos, rot, info, state, nbIn, bonds, hi);
        const Imager IM(P, a.pos, SC_BINNED_P);
        const int k = claim_rule(P, a, b, IM(b.pos) - a.pos, step);
        if (k >= 0 && pnb < SC_MAX_ACTIVE_INTERACTIONS) {
            const sc_rule &pii = P.prules[k];
            int *pb = bonds + (size_t)i * 24;
            pb[3 * pnb] = pii.id;
            pb[3 * pnb + 1] = pii.group;
            pb[3 * pnb + 2] = i == lo ? b.id : a.id;
            pnb++;
        }
    }
    nbOut[i] = pnb;
  }
}

// ---- interactions.cuh:349-555 transitionInteractions -------------------------
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_transition(
    ScParams P, const uint32_t *__restrict__ cellStart, const int *__restrict__ nActivePtr,
    const int *__restrict__ stepPtr, const float4 *__restrict__ pos, const float4 *__restrict__ rot,
    const int4 *__restrict__ info, const int *__restrict__ stateIn, int *__restrict__ stateOut, const int *__restrict__ nbIn,
    int *__restrict__ nbOut, const int *__restrict__ bondsIn, int *__restrict__ bondsOut, int *lscs, int *spoly) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    const int step = *stepPtr;
    int4 in = info[i];
    rep_apply<BATCH>(P, in.w);
    int pnb = min(max(nbIn[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
    int pstate = stateIn[i];
    int b[SC_MAX_ACTIVE_INTERACTIONS * 3];
#pragma unroll
    for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS * 3; k++) b[k] = k < 3 * pnb ? bondsIn[(size_t)i * 24 + k] : 0;
    // Only bonds whose rule transitions or breaks after a transition act in
    // the scan: without one the scan would change nothing.
    bool acts = false;
#pragma unroll
    for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++)
        if (k < pnb && b[3 * k] >= 10) {
            const sc_rule &pii = rule_at(P, b[3 * k]);
            acts |= pii.transition_to >= 0 || pii.break_after_transition;
        }
    if ((in.z & SC_ACTIVE) && acts) {
        float4 p4 = pos[i];
        const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, ppos, SC_BINNED_P);
        const sc_f4 prot = ld4(rot, i);
        const int pid = in.x, ptype = in.y;
        const sc_f3 up = sc_rotate(sc_up(), prot);
        int src = -1;
        int tId = 0, tGroup = 0, tSet = 0, tFirst = 0, tSecond = 0, tFs = 0, tSs = 0, tPoly = 0;
        const float lim = P.maxInt;
        scan27(P, cellStart, ppos, reach(P, ppos, lim, SC_BINNED_P), [&](int j) {
            if (j == i) return;
            float4 t4 = pos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - ppos;
            if (outside_cube(delta, lim)) return;
            int4 tin = info[j];
            if (!(tin.z & SC_ACTIVE)) return;
            bool loaded = false;
            sc_f4 trot;
            sc_f3 tup;
            const int ttype = tin.y;
            const bool ord = p_order(ptype, pid, ttype, tin.x);
            for (int k = 0; k < pnb; k++) {
                if (b[3 * k] < 10) continue;
                if (b[3 * k + 2] != tin.x) continue;
                const sc_rule &pii = rule_at(P, b[3 * k]);
                if (!(pii.transition_to >= 0 || pii.break_after_transition)) continue;
                if (!loaded) { trot = ld4(rot, j); tup = sc_rotate(sc_up(), trot); loaded = true; }
                float oa, rpa;
                alignment(ord, prot, trot, up, tup, delta, pii, &oa, &rpa);
                bool aligned = pii.break_after_transition || !pii.wait_for_alignment ||
                               (oa > pii.orientation_alignment_threshold &&
                                fabs((double)rpa - 1.0) < (1.0 - (double)pii.position_alignment_threshold));
                if (!(aligned && (!pii.wait_for_state || states_match(ord, pstate, stateIn[j], pii)))) continue;
                if (pii.transition_to >= 0) {
                    const sc_rule &tpii = rule_at(P, pii.transition_to);
                    if (tpii.group >= 0 && tpii.group != pii.group) {
                        bool ga = false;
                        for (int l = 0; l < pnb; l++)
                            if (b[3 * l + 1] == tpii.group) { ga = true; break; }
                        if (!ga) ga = group_active_in(bondsIn + (size_t)j * 24, nbIn[j], tpii.group);
                        if (ga) continue;
                    }
                    if (!tpii.set_state || !((ptype == tpii.first_partner_type && tpii.first_partner_state >= 0) ||
                                             (ptype == tpii.second_partner_type && tpii.second_partner_state >= 0))) {
                        b[3 * k] = tpii.id;
                        b[3 * k + 1] = tpii.group;
                    } else {
                        src = k;
                        tId = tpii.id; tGroup = tpii.group; tSet = tpii.set_state;
                        tFirst = tpii.first_partner_type; tSecond = tpii.second_partner_type;
                        tFs = tpii.first_partner_state; tSs = tpii.second_partner_state; tPoly = tpii.polymerize;
                    }
                } else if (pii.break_after_transition) {
                    for (int l = k; l < pnb - 1; l++) {
                        b[3 * l] = b[3 * l + 3];
                        b[3 * l + 1] = b[3 * l + 4];
                        b[3 * l + 2] = b[3 * l + 5];
                    }
                    pnb--;
                    if (src > k) src--;
                    k--;
                }
            }
        });
        if (src >= 0) {
            b[3 * src] = tId;
            b[3 * src + 1] = tGroup;
            if (tSet) {
                if (ptype == tFirst && tFs >= 0) { pstate = tFs; lscs[i] = step; }
                if (ptype == tSecond && tSs >= 0) { pstate = tSs; lscs[i] = step; }
            }
            if (tPoly >= 0) {
                const sc_rule &poly = rule_at(P, tPoly);
                if (poly.first_partner_type == ptype || poly.second_partner_type == ptype) spoly[i] = tPoly;
            }
        }
    }
    stateOut[i] = pstate;
    nbOut[i] = pnb;
    for (int k = 0; k < 3 * pnb; k++) bondsOut[(size_t)i * 24 + k] = b[k];
}

// ---- interactions.cuh:558-740 polymerize --------------------------------------
// The reference runs it in place with atomicAdd slot / id allocation and
// cross-slot writes, so its outcome depends on thread scheduling.  Here the
// outcome is the one a one-item-at-a-time execution in slot (index) order
// gives, computed in parallel:
//  * k_poly_count / k_poly_offsets / k_poly_plan list the scheduled items in
//    index order (an ordered compaction), with the rank of each one's new
//    monomer among the items whose rule creates one: in slot order the k-th
//    creating item takes index lastActive + 1 + k and id nextId + k (when
//    the index is below the capacity), so neither needs a serial counter;
//  * an item's processing reads and writes its own bonds and those of its
//    previous monomer (pmi, found by id among the binned particles, whose
//    ids no processing changes) and writes its new monomer's slot.  When no
//    listed item's previous monomer is itself listed or shared with another
//    item, the footprints are disjoint and every item runs at once
//    (k_poly_apply); otherwise one thread runs them all in slot order
//    (k_poly_finish), as before.
__device__ __forceinline__ bool poly_scheduled(const PFields &F, int n0, int i) {
    return i < n0 && (F.info[i].z & SC_ACTIVE) && F.spoly[i] >= 0;
}
__device__ __forceinline__ bool poly_creates(const ScParams &P, const PFields &F, int i) {
    const sc_rule &poly = rule_at(P, F.spoly[i]);
    const bool first = poly.first_partner_type == F.info[i].y;
    return (first ? poly.second_partner_type : poly.first_partner_type) >= 0;
}
// First bond of the rule's group (the active polymerisation bond), -1 if none.
__device__ __forceinline__ int poly_api(const sc_rule &poly, const int *pb, int pnb) {
    for (int k = 0; k < pnb; k++)
        if (pb[3 * k + 1] == poly.group) return k;
    return -1;
}
// The binned particle whose id is `target` (the last one in scan order).
__device__ __forceinline__ int poly_find(const ScParams &P, const uint32_t *cellStart, const PFields &F, int i,
                                         int target) {
    float4 p4 = F.pos[i];
    int pmi = -1;
    scan27(P, cellStart, sc_make_f3(p4.x, p4.y, p4.z), [&](int j) {
        if (j == i) return;
        int4 tin = F.info[j];
        if (!(tin.z & SC_ACTIVE)) return;
        if (tin.x == target) pmi = j;
    });
    return pmi;
}

// Removes the first bond of `group` from item m's bonds (shifting the rest).
__device__ __forceinline__ int poly_drop_group(int *mb, int mnb, int group) {
    for (int k = 0; k < mnb; k++) {
        if (mb[3 * k + 1] == group) {
            for (int l = k; l < mnb - 1; l++) {
                mb[3 * l] = mb[3 * l + 3]; mb[3 * l + 1] = mb[3 * l + 4]; mb[3 * l + 2] = mb[3 * l + 5];
            }
            return mnb - 1;
        }
    }
    return mnb;
}

// One scheduled item: `pmi` its previous monomer (-2: find it now), its new
// monomer at newIdx with id newId (used when newIdx < N).
__device__ void poly_one(const ScParams &P, const uint32_t *cellStart, const PFields &F, int i, int step, int pmi,
                         int newIdx, int newId) {
    int4 in = F.info[i];
    const sc_rule &poly = rule_at(P, F.spoly[i]);
    const int pid = in.x, ptype = in.y;
    int *pb = F.bonds + (size_t)i * 24;
    int pnb = min(max(F.nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
    const int api = poly_api(poly, pb, pnb);
    if (pmi == -2) pmi = api >= 0 ? poly_find(P, cellStart, F, i, pb[3 * api + 2]) : -1;
    float4 p4 = F.pos[i];
    const sc_f3 ppos = sc_make_f3(p4.x, p4.y, p4.z);
    const bool first = poly.first_partner_type == ptype;
    const int newType = first ? poly.second_partner_type : poly.first_partner_type;
    const int newState = first ? poly.second_partner_state : poly.first_partner_state;
    const int spolyId = F.spoly[i];
    if (newType >= 0) {
        float nr = 0.0f;
        int nh = 0;
        if (newType < P.nTypes) { nr = P.types[newType].radius; nh = P.types[newType].hydrophobic; }
        if (newIdx < P.N) {
            sc_f3 rp = rule_pos(poly);
            sc_f4 ro = rule_ori(poly);
            sc_f4 prot = ld4(F.rot, i);
            sc_f3 npos = ppos + sc_rotate(ptype < newType ? rp : -rp, prot);
            if (P.periodic) npos = sc_wrap3(npos, P.simSize);
            sc_f4 nrot = sc_qmul(prot, ptype < newType ? ro : sc_qinv(ro));
            // Particle(newId, newType, 0, radius, hydrophobic, pos, rot): types.cuh:192-221
            F.pos[newIdx] = make_float4(npos.x, npos.y, npos.z, nr);
            F.vel[newIdx] = make_float4(0, 0, 0, 0);
            st4(F.rot, newIdx, nrot);
            F.angvel[newIdx] = make_float4(0, 0, 0, 1);
            F.posnoise[newIdx] = make_float4(0, 0, 0, 0);
            F.angnoise[newIdx] = make_float4(0, 0, 0, 1);
            F.dbg[newIdx] = make_float4(0, 0, 0, 0);
            F.info[newIdx] = make_int4(newId, newType, SC_ACTIVE, (int)(int8_t)nh);
            F.state[newIdx] = newState >= 0 ? newState : 0;
            F.lscs[newIdx] = newState >= 0 ? step : -1;
            F.spoly[newIdx] = -1;
            int *nbp = F.bonds + (size_t)newIdx * 24;
            int nnb = 0;
            nbp[0] = spolyId; nbp[1] = poly.group; nbp[2] = pid;
            nnb = 1;
            if (pmi >= 0) {
                int *mb = F.bonds + (size_t)pmi * 24;
                int mnb = poly_drop_group(mb, min(max(F.nb[pmi], 0), SC_MAX_ACTIVE_INTERACTIONS), poly.group);
                if (mnb < SC_MAX_ACTIVE_INTERACTIONS) {
                    mb[3 * mnb] = SC_INTERACTION_TYPE_CHAIN; mb[3 * mnb + 1] = SC_INTERACTION_GROUP_FORWARD;
                    mb[3 * mnb + 2] = newId;
                }
                mnb++;
                F.nb[pmi] = mnb;
                nbp[3] = SC_INTERACTION_TYPE_CHAIN; nbp[4] = SC_INTERACTION_GROUP_BACKWARD; nbp[5] = F.info[pmi].x;
                nnb = 2;
                pb[3 * api] = spolyId;
                pb[3 * api + 2] = newId;
            } else {
                if (pnb < SC_MAX_ACTIVE_INTERACTIONS) {
                    pb[3 * pnb] = spolyId; pb[3 * pnb + 1] = poly.group; pb[3 * pnb + 2] = newId;
                }
                pnb++;
            }
            for (int k = 3 * nnb; k < 24; k++) nbp[k] = 0;
            F.nb[newIdx] = nnb;
        }
    } else {
        // End of the chain; the reference's out-of-bounds stores without a
        // previous monomer / active bond (interactions.cuh:728, 731-734) are skipped.
        if (pmi >= 0) {
            int *mb = F.bonds + (size_t)pmi * 24;
            F.nb[pmi] = poly_drop_group(mb, min(max(F.nb[pmi], 0), SC_MAX_ACTIVE_INTERACTIONS), poly.group);
        }
        if (api >= 0) {
            for (int l = api; l < pnb - 1; l++) {
                pb[3 * l] = pb[3 * l + 3]; pb[3 * l + 1] = pb[3 * l + 4]; pb[3 * l + 2] = pb[3 * l + 5];
            }
            pnb--;
        }
    }
    F.nb[i] = pnb;
    F.spoly[i] = -1;
}

// Per block of SC_THREADS items: (scheduled, creating) counts.
__global__ void __launch_bounds__(SC_THREADS) k_poly_count(ScParams P, PFields F, const ScCounters *ctr,
                                                           int2 *blk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n0 = ctr->nActive;
    const bool s = poly_scheduled(F, n0, i);
    const bool c = s && poly_creates(P, F, i);
    const int ns = __syncthreads_count(s), nc = __syncthreads_count(c);
    if (threadIdx.x == 0) blk[blockIdx.x] = make_int2(ns, nc);
}

// Exclusive offsets of the block counts (one CTA), the totals, and the
// conflict flag cleared.
#define SC_POLY_SCAN_THREADS 1024
__global__ void __launch_bounds__(SC_POLY_SCAN_THREADS) k_poly_offsets(const int2 *__restrict__ blk, int2 *off,
                                                                       int nblk, ScCounters *ctr) {
    __shared__ int2 s_w[SC_POLY_SCAN_THREADS / 32];
    __shared__ int2 s_carry;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_carry = make_int2(0, 0);
    __syncthreads();
    for (int b0 = 0; b0 < nblk; b0 += SC_POLY_SCAN_THREADS) {
        const int b = b0 + t;
        const int2 v = b < nblk ? blk[b] : make_int2(0, 0);
        int2 x = v;  // inclusive warp scan
        for (int d = 1; d < 32; d *= 2) {
            const int ax = __shfl_up_sync(0xffffffffu, x.x, d), ay = __shfl_up_sync(0xffffffffu, x.y, d);
            if (lane >= d) { x.x += ax; x.y += ay; }
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int2 w = s_w[lane];
            for (int d = 1; d < 32; d *= 2) {
                const int ax = __shfl_up_sync(0xffffffffu, w.x, d), ay = __shfl_up_sync(0xffffffffu, w.y, d);
                if (lane >= d) { w.x += ax; w.y += ay; }
            }
            s_w[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const int2 before = warp ? s_w[warp - 1] : make_int2(0, 0);
        const int2 carry = s_carry;
        if (b < nblk) off[b] = make_int2(carry.x + before.x + x.x - v.x, carry.y + before.y + x.y - v.y);
        __syncthreads();
        if (t == 0) s_carry = make_int2(carry.x + s_w[31].x, carry.y + s_w[31].y);
        __syncthreads();
    }
    if (t == 0) {
        ctr->polyCount = s_carry.x;
        ctr->polyCreates = s_carry.y;
        ctr->polyConflict = 0;
    }
}

// Lists the scheduled items in index order with their monomer ranks, finds
// each one's previous monomer, and flags a conflict when a previous monomer
// is itself scheduled or claimed by two items.
__global__ void __launch_bounds__(SC_THREADS) k_poly_plan(ScParams P, const uint32_t *__restrict__ cellStart, PFields F,
                                                          ScCounters *ctr, const int2 *__restrict__ off, int *list,
                                                          int *rank, int *pmiOut, int *claim) {
    __shared__ int2 s_w[SC_THREADS / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int n0 = ctr->nActive;
    const bool s = poly_scheduled(F, n0, i);
    const bool c = s && poly_creates(P, F, i);
    const unsigned bs = __ballot_sync(0xffffffffu, s), bc = __ballot_sync(0xffffffffu, c);
    const unsigned below = (1u << lane) - 1u;
    if (lane == 0) s_w[warp] = make_int2(__popc(bs), __popc(bc));
    __syncthreads();
    if (!s) return;
    int2 o = off[blockIdx.x];
    for (int w = 0; w < warp; w++) { o.x += s_w[w].x; o.y += s_w[w].y; }
    const int slot = o.x + __popc(bs & below);
    list[slot] = i;
    rank[slot] = c ? o.y + __popc(bc & below) : -1;
    const sc_rule &poly = rule_at(P, F.spoly[i]);
    const int *pb = F.bonds + (size_t)i * 24;
    const int api = poly_api(poly, pb, min(max(F.nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS));
    const int pmi = api >= 0 ? poly_find(P, cellStart, F, i, pb[3 * api + 2]) : -1;
    pmiOut[slot] = pmi;
    if (pmi >= 0 && (poly_scheduled(F, n0, pmi) || atomicAdd(&claim[pmi], 1) != 0)) ctr->polyConflict = 1;
}

// Without a conflict every listed item runs at once; either way the claims
// are cleared for the next step.
__global__ void __launch_bounds__(SC_THREADS) k_poly_apply(ScParams P, const uint32_t *__restrict__ cellStart, PFields F,
                                                           const ScCounters *ctr, const int *__restrict__ list,
                                                           const int *__restrict__ rank, const int *__restrict__ pmiIn,
                                                           int *claim) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= ctr->polyCount) return;
    const int pmi = pmiIn[slot];
    if (pmi >= 0) claim[pmi] = 0;
    if (ctr->polyConflict) return;
    const int r = rank[slot];
    poly_one(P, cellStart, F, list[slot], ctr->step, pmi, r >= 0 ? ctr->lastActive + 1 + r : P.N,
             r >= 0 ? ctr->nextId + r : -1);
}

// The serial path of a conflicting list, then the counters: lastActive
// advances by every creating item (the reference increments it before its
// capacity test), nextId and nActive by those that fit.
__global__ void k_poly_finish(ScParams P, const uint32_t *__restrict__ cellStart, PFields F, ScCounters *ctr,
                              const int *__restrict__ list, const int *__restrict__ rank) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int count = ctr->polyCount;
    if (count == 0) return;
    const int last0 = ctr->lastActive, next0 = ctr->nextId;
    if (ctr->polyConflict) {
        for (int k = 0; k < count; k++) {
            const int r = rank[k];
            poly_one(P, cellStart, F, list[k], ctr->step, -2, r >= 0 ? last0 + 1 + r : P.N, r >= 0 ? next0 + r : -1);
        }
    }
    const int R = ctr->polyCreates;
    const int made = max(0, min(R, P.N - 1 - last0));
    ctr->lastActive = last0 + R;
    ctr->nextId = next0 + made;
    ctr->nActive += made;
    ctr->polyCount = 0;
}

// ---- interactions.cuh:743-822 propagateState (sc_config.propagate_state) -----
// The reference's kernel, whose launch its step leaves commented out
// (main.cu:618-631); it runs after polymerize when the config asks for it.
// Each active particle below the count after polymerize walks its 27 cells in
// order and, for every active neighbour inside the interaction cube that is
// the partner of one of its rule bonds (type >= 10) whose rule sets
// propagateState, takes the neighbour's state and last state-change step when
// that step is later than its own as updated so far.  Neighbours are read
// from the state before the pass (state and lscs are double-buffered).  A
// particle without such a bond keeps its state and scans nothing.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_propagate_state(
    ScParams P, const uint32_t *__restrict__ cellStart, const int *__restrict__ nActivePtr,
    const float4 *__restrict__ pos, const int4 *__restrict__ info, const int *__restrict__ stateIn,
    int *__restrict__ stateOut, const int *__restrict__ lscsIn, int *__restrict__ lscsOut, const int *__restrict__ nb,
    const int *__restrict__ bonds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    const int4 in = info[i];
    int st = stateIn[i], ls = lscsIn[i];
    const int pnb = min(max(nb[i], 0), SC_MAX_ACTIVE_INTERACTIONS);
    int partner[SC_MAX_ACTIVE_INTERACTIONS];
    unsigned prop = 0u;  // bit k: bond k propagates
#pragma unroll
    for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++) {
        const int t = k < pnb ? bonds[(size_t)i * 24 + 3 * k] : 0;
        partner[k] = k < pnb ? bonds[(size_t)i * 24 + 3 * k + 2] : 0;
        if (k < pnb && t >= 10 && rule_at(P, t).propagate_state) prop |= 1u << k;
    }
    if ((in.z & SC_ACTIVE) && prop) {
        rep_apply<BATCH>(P, in.w);
        const float4 p4 = pos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_P);
        scan27(P, cellStart, pp, [&](int j) {
            if (j == i) return;
            const int4 tin = info[j];
            if (!(tin.z & SC_ACTIVE)) return;
            const float4 t4 = pos[j];
            const sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, P.maxInt)) return;
#pragma unroll
            for (int k = 0; k < SC_MAX_ACTIVE_INTERACTIONS; k++) {
                if (((prop >> k) & 1u) && partner[k] == tin.x) {
                    const int tl = lscsIn[j];
                    if (tl > ls) {
                        ls = tl;
                        st = stateIn[j];
                    }
                }
            }
        });
    }
    stateOut[i] = st;
    lscsOut[i] = ls;
}

// ---- metabolites.cuh:352-431 diffuseMetabolites ------------------------------
// List: the metabolic items within maxDiffusionDistance (cube, then sphere),
// built after applyVelocities and read by all diffusion sub-iterations.
__device__ __forceinline__ void build_d_item(const ScParams &P, const uint32_t *__restrict__ cellStart, int i,
                                             const float4 *__restrict__ pos, const int4 *__restrict__ info,
                                             uint32_t *list, int &c) {
    float4 p4 = pos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_M);
    const float lim = P.maxDiff;
    const sc_sqrt_le within = sc_sqrt_le_make(lim);
    scan27(P, cellStart, pp, reach(P, pp, lim, SC_BINNED_M), [&](int j) {
        if (j == i || !active_m(P, info, j)) return;
        float4 t4 = pos[j];
        sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
        if (outside_cube(delta, lim)) return;
        if (sc_sqrt_le_test(within, sc_normsq3(delta))) {
            if (c < min(SC_LIST_D, P.listLimit)) list[sc_list_at(SC_LIST_D, i, c)] = (uint32_t)j;
            c++;
        }
    });
}

template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_d(ScParams P, const uint32_t *__restrict__ cellStart,
                                                        const int *__restrict__ nActivePtr,
                                                        const float4 *__restrict__ pos, const int4 *__restrict__ info,
                                                        uint32_t *__restrict__ list, uint32_t *scratch,
                                                        int *__restrict__ cnt, int *__restrict__ perm, int cap,
                                                        int *__restrict__ ovf, int *__restrict__ ovfCount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < *nActivePtr;
    int c = 0;
    if (valid) {
        const int4 in = info[i];
        ScParams Q = P;
        rep_apply<BATCH>(Q, in.w);
        if (in.z & SC_ACTIVE) build_d_item(Q, cellStart, i, pos, info, scratch, c);
    }
    emit_count_ordered<SC_LIST_D>(valid, c, P.listLimit, cap, scratch, list, cnt, perm, ovf, ovfCount);
}

// The full diffusion lists of the overflowed positions (listed by k_build_d;
// their counts are in cnt): each takes a contiguous region of the overflow
// pool by atomicAdd and writes its neighbours there in build_d_item's order,
// for k_diffuse_pool; a position the pool has no room for keeps offset -1 (it
// scans).  The demand is counted in full for the pool's growth at the next
// synchronisation.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_build_d_ovf(ScParams P0, const uint32_t *__restrict__ cellStart,
                                                            const float4 *__restrict__ pos,
                                                            const int4 *__restrict__ info, const int *__restrict__ ovf,
                                                            const int *__restrict__ ovfCount, const int *__restrict__ cnt,
                                                            const int *__restrict__ perm, long long *__restrict__ ovfOff,
                                                            uint32_t *__restrict__ pool, long long cap,
                                                            unsigned long long *__restrict__ demand) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < *ovfCount; t += gridDim.x * blockDim.x) {
        const int g = ovf[t], i = perm[g], n = cnt[g];
        // regions start on 16-byte boundaries (whole chunks of four entries)
        const unsigned long long n4 = (unsigned long long)((n + 3) & ~3);
        const unsigned long long base = n > 0 ? atomicAdd(demand, n4) : 0ull;
        if (i < 0 || n <= 0 || base + n4 > (unsigned long long)cap) {
            ovfOff[g] = -1;
            continue;
        }
        ovfOff[g] = (long long)base;
        ScParams P = P0;
        rep_apply<BATCH>(P, info[i].w);
        const float4 p4 = pos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_M);
        const float lim = P.maxDiff;
        const sc_sqrt_le within = sc_sqrt_le_make(lim);
        uint32_t *out = pool + base;
        int k = 0;
        scan27(P, cellStart, pp, reach(P, pp, lim, SC_BINNED_M), [&](int j) {
            if (j == i || !active_m(P, info, j)) return;
            const float4 t4 = pos[j];
            const sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) return;
            if (sc_sqrt_le_test(within, sc_normsq3(delta)) && k < n) out[k++] = (uint32_t)j;
        });
    }
}

// An item's amounts, Q float4 per item: eight-amount rows (32 bytes,
// aligned) in one access.
template <int Q>
__device__ __forceinline__ void met_row(const float4 *__restrict__ met, int j, float4 (&v)[Q]) {
    if (Q == 2) {
        ld_row8(met + (size_t)j * 2, v[0], v[1]);
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) v[q] = met[(size_t)j * Q + q];
    }
}
template <int SP>
__device__ __forceinline__ void met_store(float4 *__restrict__ met, int i, const float (&pm)[SP]) {
    if (SP == 8) {
        st_row8(met + (size_t)i * 2, make_float4(pm[0], pm[1], pm[2], pm[3]), make_float4(pm[4], pm[5], pm[6], pm[7]));
    } else {
#pragma unroll
        for (int q = 0; q < SP / 4; q++)
            met[(size_t)i * (SP / 4) + q] = make_float4(pm[4 * q], pm[4 * q + 1], pm[4 * q + 2], pm[4 * q + 3]);
    }
}
// One neighbour's amounts against the item's, the first S of SP amounts
// (metabolites.cuh:352-431, the exchange of one pair).
template <int SP>
__device__ __forceinline__ void diffuse_term(const float4 (&v)[SP / 4], const float (&pm)[SP], float (&dm)[SP],
                                             int S) {
#pragma unroll
    for (int q = 0; q < SP / 4; q++) {
        const float tm[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = 4 * q + c;
            if (k < S) {
                const float diff = tm[c] - pm[k];
                if (sc_diffuse_exceeds(diff)) dm[k] += diff * 0.1f;
            }
        }
    }
}

template <int SP, bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_diffuse(ScParams P, const uint32_t *__restrict__ cellStart,
                                                        const int *__restrict__ nActivePtr,
                                                        const float4 *__restrict__ pos, const int4 *__restrict__ info,
                                                        PairList<SC_LIST_D> L, const float4 *__restrict__ metIn,
                                                        float4 *__restrict__ metOut, const long long *__restrict__ ovfOff,
                                                        const uint32_t *__restrict__ ovfPool) {
    constexpr int Q = SP / 4;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;   // list position (count-ordered)
    if (g >= *nActivePtr) return;
    const int i = L.perm[g];
    if (i < 0) return;
    if (BATCH) rep_apply<BATCH>(P, info[i].w);
    float pm[SP];
    {
        float4 v[Q];
        met_row<Q>(metIn, i, v);
#pragma unroll
        for (int q = 0; q < Q; q++) {
            pm[4 * q] = v[q].x; pm[4 * q + 1] = v[q].y; pm[4 * q + 2] = v[q].z; pm[4 * q + 3] = v[q].w;
        }
    }
    // after the sort the active items are exactly the binned ones
    const bool act = P.mAllActive ? i < (int)cellStart[P.cells] : (info[i].z & SC_ACTIVE) != 0;
    if (!act) {
        met_store<SP>(metOut, i, pm);   // the amounts' bits, unchanged
        return;
    }
    float dm[SP];
#pragma unroll
    for (int k = 0; k < SP; k++) dm[k] = 0.0f;
    const int S = P.S;
    const int c = L.cnt[g];
    if (c <= min(SC_LIST_D, P.listLimit)) {
        // four entries per list load; their amounts are gathered together and
        // the next chunk of the list is loaded while this one is applied
        const uint4 *__restrict__ chunks = sc_list4_chunks(L.list, SC_LIST_D, g);
        uint4 E = c > 0 ? chunks[0] : make_uint4(0, 0, 0, 0);
        for (int k0 = 0; k0 < c; k0 += 4) {
            const uint4 En = k0 + 4 < c ? chunks[(size_t)(k0 / 4 + 1) * 32] : make_uint4(0, 0, 0, 0);
            const int e[4] = {(int)E.x, (int)E.y, (int)E.z, (int)E.w};
            float4 v[4][Q];
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                if (k0 + kk < c) met_row<Q>(metIn, e[kk], v[kk]);
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                if (k0 + kk >= c) break;
                diffuse_term<SP>(v[kk], pm, dm, S);
            }
            E = En;
        }
    } else if (ovfOff && ovfOff[g] >= 0) {
        return;   // an overflowed list kept whole in the overflow pool: k_diffuse_pool
    } else {
        float4 p4 = pos[i];
        const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
        const Imager IM(P, pp, SC_BINNED_M);
        const float lim = P.maxDiff;
        const sc_sqrt_le within = sc_sqrt_le_make(lim);
        scan27(P, cellStart, pp, reach(P, pp, lim, SC_BINNED_M), [&](int j) {
            if (j == i) return;
            if (!active_m(P, info, j)) return;
            float4 t4 = pos[j];
            sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
            if (outside_cube(delta, lim)) return;
            if (sc_sqrt_le_test(within, sc_normsq3(delta))) {
                float4 v[Q];
                met_row<Q>(metIn, j, v);
                diffuse_term<SP>(v, pm, dm, S);
            }
        });
    }
#pragma unroll
    for (int k = 0; k < SP; k++)
        if (k < S) pm[k] += dm[k];
    met_store<SP>(metOut, i, pm);
}

// The positions whose overflowed list is kept whole in the overflow pool
// (k_build_d_ovf), one warp per position: the lanes gather 32 neighbours'
// amounts at once and each computes its neighbour's terms (zero where the
// threshold drops the pair; a kept term is never zero), then lane k adds the
// kept terms of amount k in list order from shared memory -- the sums a
// thread walking the list forms, term by term, while the list's pile-sized
// length costs one gather latency per 32 neighbours instead of per 4.
template <int SP>
__global__ void __launch_bounds__(SC_THREADS) k_diffuse_pool(ScParams P, const int4 *__restrict__ info,
                                                             PairList<SC_LIST_D> L, const int *__restrict__ ovf,
                                                             const int *__restrict__ ovfCount,
                                                             const long long *__restrict__ ovfOff,
                                                             const uint32_t *__restrict__ ovfPool,
                                                             const float4 *__restrict__ metIn,
                                                             float4 *__restrict__ metOut) {
    constexpr int Q = SP / 4;
    __shared__ float sTerm[SC_THREADS / 32][32][SP + 1];   // odd row length: no bank conflicts either way
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int S = P.S;
    const int n = *ovfCount;
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n; t += (gridDim.x * blockDim.x) >> 5) {
        const int g = ovf[t];
        const long long off = ovfOff[g];
        const int i = L.perm[g];
        if (off < 0 || i < 0) continue;   // scanned by k_diffuse
        float pm[SP];
        {
            float4 v[Q];
            met_row<Q>(metIn, i, v);
#pragma unroll
            for (int q = 0; q < Q; q++) {
                pm[4 * q] = v[q].x; pm[4 * q + 1] = v[q].y; pm[4 * q + 2] = v[q].z; pm[4 * q + 3] = v[q].w;
            }
        }
        // lane k's amount and its running sum
        float mine = 0.0f, dm = 0.0f;
#pragma unroll
        for (int k = 0; k < SP; k++)
            if (lane == k) mine = pm[k];
        if (info[i].z & SC_ACTIVE) {
            const int c = L.cnt[g];
            const uint32_t *__restrict__ e = ovfPool + off;
            for (int b = 0; b < c; b += 32) {
                float term[SP];
#pragma unroll
                for (int k = 0; k < SP; k++) term[k] = 0.0f;
                if (b + lane < c) {
                    float4 v[Q];
                    met_row<Q>(metIn, (int)e[b + lane], v);
#pragma unroll
                    for (int q = 0; q < Q; q++) {
                        const float tm[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
                        for (int cc = 0; cc < 4; cc++) {
                            const int k = 4 * q + cc;
                            const float diff = tm[cc] - pm[k];
                            if (k < S && sc_diffuse_exceeds(diff)) term[k] = diff * 0.1f;
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < SP; k++) sTerm[wid][lane][k] = term[k];
                __syncwarp();
                if (lane < S) {
                    const int m = min(32, c - b);
                    for (int u = 0; u < m; u++) {
                        const float x = sTerm[wid][u][lane];
                        if (x != 0.0f) dm += x;
                    }
                }
                __syncwarp();
            }
            if (lane < S) mine += dm;
        }
        if (lane < SP) reinterpret_cast<float *>(metOut)[(size_t)i * SP + lane] = mine;
    }
}

// ---- metabolites.cuh:18-88 removeInterferingMetabolicParticles -------------
// Only the item's own flags change and no other thread reads metabolic
// flags here: updated in place.
template <bool BATCH>
__global__ void __launch_bounds__(SC_THREADS) k_remove_interfering(
    ScParams P, const uint32_t *__restrict__ cellStartP, const int *__restrict__ nActivePtr,
    const float4 *__restrict__ mpos, int4 *__restrict__ minfo, const float4 *__restrict__ ppos_,
    const int4 *__restrict__ pinfo) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nActivePtr) return;
    int4 in = minfo[i];
    if (!(in.z & SC_ACTIVE)) return;
    rep_apply<BATCH>(P, in.w);
    float4 p4 = mpos[i];
    const sc_f3 pp = sc_make_f3(p4.x, p4.y, p4.z);
    const Imager IM(P, pp, SC_BINNED_P);
    const float prad = p4.w;
    int flags = in.z;
    const float lim = P.maxInt;
    scan27(P, cellStartP, pp, reach(P, pp, lim, SC_BINNED_P), [&](int j) {
        if (!active_lipid(P, pinfo, j)) return;
        float4 t4 = ppos_[j];
        sc_f3 delta = IM(sc_make_f3(t4.x, t4.y, t4.z)) - pp;
        if (outside_cube(delta, lim)) return;
        float dist = sc_norm3(delta);
        float interf = (float)((double)(prad + t4.w) + 0.001);
        if (dist <= interf) flags = flags & ~SC_ACTIVE;
    });
    if (flags != in.z) minfo[i].z = flags;
}

// ---- dynamics.cuh:824-844 reduceParticles (frames.dat records) --------------
__device__ __forceinline__ void reduce_common(sc_reduced_particle &r, int4 in, int state, float4 p4, float4 r4,
                                              float4 d4) {
    r.id = in.x;
    r.type = in.y;
    r.flags = in.z | (((int)(int8_t)state & 0x0000000F) << 16);
    r.radius = sc_f2h(p4.w);
    r.pos[0] = sc_f2h(p4.x); r.pos[1] = sc_f2h(p4.y); r.pos[2] = sc_f2h(p4.z);
    r.rot[0] = sc_f2h(r4.x); r.rot[1] = sc_f2h(r4.y); r.rot[2] = sc_f2h(r4.z); r.rot[3] = sc_f2h(r4.w);
    r.debug_vector[0] = sc_f2h(d4.x); r.debug_vector[1] = sc_f2h(d4.y);
    r.debug_vector[2] = sc_f2h(d4.z); r.debug_vector[3] = sc_f2h(d4.w);
}

__global__ void __launch_bounds__(SC_THREADS) k_reduce_particles(const int *__restrict__ nActivePtr, int cap,
                                                                 PFields F, sc_reduced_particle *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    sc_reduced_particle r;
    memset(&r, 0, sizeof r);
    if (i < *nActivePtr) reduce_common(r, F.info[i], F.state[i], F.pos[i], F.rot[i], F.dbg[i]);
    out[i] = r;
}

__global__ void __launch_bounds__(SC_THREADS) k_reduce_metabolic(const int *__restrict__ nActivePtr, int cap, int sp4,
                                                                 MFields F, sc_reduced_metabolic_particle *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    sc_reduced_metabolic_particle r;
    memset(&r, 0, sizeof r);
    if (i < *nActivePtr) {
        reduce_common(r.p, F.info[i], F.state[i], F.pos[i], F.rot[i], F.dbg[i]);
        float4 m = F.met[(size_t)i * sp4];
        r.metabolites[0] = sc_f2h(m.x); r.metabolites[1] = sc_f2h(m.y);
        r.metabolites[2] = sc_f2h(m.z); r.metabolites[3] = sc_f2h(m.w);
    }
    out[i] = r;
}

// ---- launchers ------------------------------------------------------------------
static inline int nblocks(int n) { return (n + SC_THREADS - 1) / SC_THREADS; }

// The instantiation of a kernel for this launch: replica-aware in batched sims.
#define SC_BATCHED(kern) (c.P.nRep > 1 ? kern<true> : kern<false>)

void sc_phase_move_brownian(ScLaunchCtx &c, bool metabolic) {
    ScBuffers &B = *c.B;
    if (!metabolic) {
        PFields F = B.P();
        if (c.P.N <= 0) return;
        SC_BATCHED(k_move_brownian)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(&B.ctr->nActive, F.info, F.pos, F.dbg, F.posnoise,
                                                                  F.angnoise, c.P, c.P.moveNoise, SC_STREAM_P_UNIFORM,
                                                                  SC_STREAM_P_NORMAL, &B.ctr->step);
    } else {
        MFields F = B.M();
        if (c.P.Nm <= 0) return;
        SC_BATCHED(k_move_brownian)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(&B.ctr->nActiveM, F.info, F.pos, F.dbg, F.posnoise,
                                                                   F.angnoise, c.P, c.P.metabNoise,
                                                                   SC_STREAM_M_UNIFORM, SC_STREAM_M_NORMAL,
                                                                   &B.ctr->step);
    }
    (*c.launches)++;
}

static void ensure_pp(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (B.validPP) return;
    PFields F = B.P();
    cudaMemsetAsync(B.ctr->ppClassCount, 0, sizeof(B.ctr->ppClassCount), c.st);
    cudaMemsetAsync(&B.ctr->ovfPP, 0, sizeof(int), c.st);
    SC_BATCHED(k_build_pp)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, &B.ctr->nActive, F.pos, F.info, F.nb,
                                                         F.bonds, B.listPP, B.cntPP, c.P.N, B.classPP,
                                                         B.ctr->ppClassCount, B.ovfPP, &B.ctr->ovfPP, B.matchPP,
                                                         B.matchN);
    (*c.launches)++;
    B.validPP = true;
}

static PairList<SC_LIST_PP> pp_list(const ScLaunchCtx &c) {
    PairList<SC_LIST_PP> L;
    L.list = c.B->listPP;
    L.cnt = c.B->cntPP;
    L.cap = c.P.N;
    L.perm = nullptr;
    return L;
}

void sc_phase_coordinate_noise(ScLaunchCtx &c, float frac) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    ensure_pp(c);
    // the other buffers of the two noise fields hold the bonded class's new
    // values by class position until they are written back in place
    PFields F = B.P(), X = B.Pnext();
    const int g = std::min(nblocks(c.P.N), c.gridCap);
    SC_BATCHED(k_coordinate_noise)<<<g, SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, B.classPP, B.ctr->ppClassCount, F.pos, F.info,
                                                    F.nb, F.bonds, pp_list(c), B.matchPP, B.matchN, F.posnoise,
                                                    F.angnoise, X.posnoise, X.angnoise, frac);
    k_noise_writeback<<<g, SC_THREADS, 0, c.st>>>(B.classPP, B.ctr->ppClassCount, X.posnoise, X.angnoise,
                                                   F.posnoise, F.angnoise);
    (*c.launches) += 2;
}

void sc_phase_apply_noise(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N > 0) {
        PFields F = B.P();
        k_apply_noise<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(&B.ctr->nActive, F.info, F.vel, F.posnoise, F.angvel,
                                                                F.angnoise);
        (*c.launches)++;
    }
    if (c.P.Nm > 0) {
        MFields M = B.M();
        k_apply_noise<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(&B.ctr->nActiveM, M.info, M.vel, M.posnoise,
                                                                 M.angvel, M.angnoise);
        (*c.launches)++;
    }
}

void sc_phase_relax(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    ensure_pp(c);
    PFields F = B.P(), X = B.Pnext();
    RelaxArgs A{B.cellStartP, &B.ctr->nActive, F.pos, F.info, F.nb, F.bonds, pp_list(c),
                F.vel, F.rot, F.angvel, X.vel, X.rot, X.angvel, F.dbg, B.classPP, B.ctr->ppClassCount,
                B.matchPP, B.matchN};
    // The three classes write disjoint items and read only the input
    // buffers: with side streams they run concurrently (bonded on st, the
    // others on the side streams), so the classes fill each other's tails;
    // each grid covers its class at most once.
    const int g = std::min(nblocks(c.P.N), c.gridCap);
    const bool fork = c.side[0] != nullptr;
    if (fork) {
        cudaEventRecord(c.fork, c.st);
        cudaStreamWaitEvent(c.side[0], c.fork, 0);
        cudaStreamWaitEvent(c.side[1], c.fork, 0);
    }
    const bool batch = c.P.nRep > 1;
    (batch ? k_relax<0, true> : k_relax<0, false>)<<<g, SC_THREADS, 0, c.st>>>(c.P, A);
    (batch ? k_relax<2, true> : k_relax<2, false>)<<<g, SC_THREADS, 0, fork ? c.side[0] : c.st>>>(c.P, A);
    (batch ? k_relax<1, true> : k_relax<1, false>)<<<g, SC_THREADS, 0, fork ? c.side[1] : c.st>>>(c.P, A);
    if (fork) {
        cudaEventRecord(c.join[0], c.side[0]);
        cudaEventRecord(c.join[1], c.side[1]);
        cudaStreamWaitEvent(c.st, c.join[0], 0);
        cudaStreamWaitEvent(c.st, c.join[1], 0);
    }
    SC_BATCHED(k_relax_overflow)<<<std::min(nblocks(c.P.N), c.gridCap / 4), SC_THREADS, 0, c.st>>>(c.P, A, B.ovfPP, &B.ctr->ovfPP);
    (*c.launches) += 3;
    B.cp[FP_VEL] ^= 1;
    B.cp[FP_ROT] ^= 1;
    B.cp[FP_ANGVEL] ^= 1;
    (*c.launches)++;
}

// Largest dynamic shared memory of the tile kernels; called once per device.
void sc_tile_init() {
    const int most = 227 * 1024;
    cudaFuncSetAttribute(k_build_m_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    cudaFuncSetAttribute(k_relax_metab_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
}
size_t sc_tile_bytes(int capM, int capP, int perSlot) { return SC_TILE_HDR_BYTES + (size_t)(capM + capP) * perSlot; }

// The metabolic relaxation's pair list (and pool) for the current
// positions, unless it is already built.
void sc_phase_build_m(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.Nm <= 0) return;
    MFields M = B.M();
    PFields F = B.P();
    const bool tiles = c.P.tileCapM > 0;
    if (!B.validM) {
        // the diffusion list's buffer is the build scratch (that list is rebuilt after the next move anyway)
        B.validD = false;
        cudaMemsetAsync(&B.ctr->ovfM, 0, sizeof(int), c.st);
        if (tiles) {
            k_build_m_tile<<<tile_blocks(c.P), SC_THREADS, sc_tile_bytes(c.P.tileCapM, c.P.tileCapP, 17), c.st>>>(
                c.P, B.cellStartM, B.cellStartP, M.pos, M.info, F.pos, F.info, reinterpret_cast<uint16_t *>(B.listM),
                B.cntM, B.ovfM, &B.ctr->ovfM);
        } else {
            cudaMemsetAsync(&B.ctr->poolM, 0, sizeof(B.ctr->poolM), c.st);
            (c.P.nRep > 1 ? (c.P.metabLean ? k_build_m<true, true> : k_build_m<false, true>)
                          : (c.P.metabLean ? k_build_m<true, false> : k_build_m<false, false>))<<<
                nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(
                c.P, B.cellStartM, B.cellStartP, &B.ctr->nActiveM, M.pos, M.info, F.pos, F.info, B.listM,
                (long long)B.poolCapM, &B.ctr->poolM, B.warpOffM, B.listD, B.cntM, B.permM, c.P.Nm, B.ovfM, &B.ctr->ovfM,
                B.ovfNM);
            // the overflowed items' full lists
            cudaMemsetAsync(&B.ctr->poolOvfM, 0, sizeof(B.ctr->poolOvfM), c.st);
            SC_BATCHED(k_build_m_ovf)<<<std::min(nblocks(c.P.Nm), c.gridCap / 4), SC_THREADS, 0, c.st>>>(
                c.P, B.cellStartM, B.cellStartP, M.pos, M.info, F.pos, F.info, B.ovfM, &B.ctr->ovfM, B.ovfNM,
                B.ovfOffM, B.ovfPoolM, (long long)B.ovfPoolCapM, &B.ctr->poolOvfM);
            (*c.launches)++;
        }
        (*c.launches)++;
        B.validM = true;
    }
}

void sc_phase_relax_metab(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.Nm <= 0) return;
    MFields M = B.M(), X = B.Mnext();
    PFields F = B.P();
    const bool tiles = c.P.tileCapM > 0;
    sc_phase_build_m(c);
    PairList<SC_LIST_M> L;
    L.list = B.listM;
    L.cnt = B.cntM;
    L.cap = c.P.Nm;
    L.perm = tiles ? nullptr : B.permM;
    RelaxMArgs A{B.cellStartM, B.cellStartP, &B.ctr->nActiveM, M.pos, M.info, L, M.vel, X.vel, F.pos, F.info, F.vel,
                 reinterpret_cast<const uint4 *>(B.listM), B.warpOffM};
    if (tiles) {
        k_relax_metab_tile<<<tile_blocks(c.P), SC_THREADS, sc_tile_bytes(c.P.tileCapM, c.P.tileCapP, 32), c.st>>>(
            c.P, A, reinterpret_cast<const uint16_t *>(B.listM), &B.ctr->error);
        k_copy_tail<<<std::max(1, c.gridCap / 8), SC_THREADS, 0, c.st>>>(
            B.cellStartM + c.P.cells, &B.ctr->nActiveM, M.vel, X.vel);
        (*c.launches) += 2;
    } else {
        (c.P.metabLean ? (c.P.nRep > 1 ? k_relax_metab_lean<true> : k_relax_metab_lean<false>) : k_relax_metab)<<<
            nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, A);
        (*c.launches)++;
    }
    SC_BATCHED(k_relax_metab_overflow)<<<std::min(nblocks(c.P.Nm), c.gridCap / 4), SC_THREADS, 0, c.st>>>(
        c.P, A, B.ovfM, &B.ctr->ovfM, B.ovfNM, tiles ? nullptr : B.ovfOffM, B.ovfPoolM);
    (*c.launches)++;
    if (!tiles) {
        k_relax_metab_pool<<<std::min(nblocks(c.P.Nm), c.gridCap), SC_THREADS, 0, c.st>>>(
            c.P, A, B.ovfM, &B.ctr->ovfM, B.ovfNM, B.ovfOffM, B.ovfPoolM);
        (*c.launches)++;
    }
    B.cm[FM_VEL] ^= 1;
}

// The lipid-metabolic pair list of relax_partners, unless it is already built.
void sc_phase_build_lm(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    MFields M = B.M();
    PFields F = B.P();
    if (!B.validLM) {
        if (B.scratchLM == B.listD) B.validD = false;
        cudaMemsetAsync(&B.ctr->poolLM, 0, sizeof(B.ctr->poolLM), c.st);
        cudaMemsetAsync(&B.ctr->workCount, 0, sizeof(int), c.st);
        k_lipid_select<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(&B.ctr->nActive, F.info, B.workP, &B.ctr->workCount);
        SC_BATCHED(k_build_lm)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(
            c.P, B.cellStartM, B.workP, &B.ctr->workCount, F.info, F.pos, M.pos, M.info,
            reinterpret_cast<uint4 *>(B.listLM),
            (long long)(sc_list_words(SC_LIST_LM, c.P.N) / 4), &B.ctr->poolLM, B.warpOffLM, B.scratchLM, B.cntLM, B.permLM,
            c.P.N);
        (*c.launches)++;
        (*c.launches)++;
        B.validLM = true;
    }
}

void sc_phase_relax_partners(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    MFields M = B.M();
    PFields F = B.P();
    sc_phase_build_lm(c);
    PairList<SC_LIST_LM> L;
    L.list = B.listLM;
    L.cnt = B.cntLM;
    L.cap = c.P.N;
    L.perm = B.permLM;
    SC_BATCHED(k_relax_partners)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(c.P, B.cellStartM, &B.ctr->nActive, F.pos, F.info,
                                                               F.vel, L, reinterpret_cast<const uint4 *>(B.listLM),
                                                               B.warpOffLM, M.pos, M.info, M.vel);
    (*c.launches)++;
}

void sc_phase_apply_velocities(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N > 0) {
        PFields F = B.P();
        SC_BATCHED(k_apply_velocities)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(&B.ctr->nActive, F.info, F.pos, F.vel, F.rot,
                                                                     F.angvel, c.P, 0.45f);
        (*c.launches)++;
    }
    if (c.P.Nm > 0) {
        MFields M = B.M();
        SC_BATCHED(k_apply_velocities)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(&B.ctr->nActiveM, M.info, M.pos, M.vel, M.rot,
                                                                      M.angvel, c.P, 0.45f);
        (*c.launches)++;
    }
}

void sc_phase_complexify(ScLaunchCtx &c, bool prep) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    PFields F = B.P(), X = B.Pnext();
    cudaMemsetAsync(&B.ctr->workCount, 0, sizeof(int), c.st);
    k_complexify_select<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(c.P, &B.ctr->nActive, F.info, F.nb, X.nb, F.bonds,
                                                                  B.workP, &B.ctr->workCount);
    const int blocks = std::min(nblocks(c.P.N), c.gridCap);
    if (!c.P.pairClaim) {
        SC_BATCHED(k_complexify)<<<blocks, SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, B.workP, &B.ctr->workCount, F.pos, F.rot,
                                                      F.info, F.state, F.nb, X.nb, F.bonds, &B.ctr->step, prep);
        (*c.launches) += 2;
    } else {
        cudaMemsetAsync(B.claimP, 0xff, (size_t)c.P.N * sizeof(unsigned long long), c.st);
        SC_BATCHED(k_claim_offer)<<<blocks, SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, B.workP, &B.ctr->workCount, F.pos, F.rot,
                                                       F.info, F.state, F.nb, F.bonds, &B.ctr->step, prep, B.claimP);
        SC_BATCHED(k_claim_bind)<<<blocks, SC_THREADS, 0, c.st>>>(c.P, B.workP, &B.ctr->workCount, F.pos, F.rot, F.info, F.state,
                                                      F.nb, X.nb, F.bonds, &B.ctr->step, prep, B.claimP);
        (*c.launches) += 3;
    }
    B.cp[FP_NB] ^= 1;
}

void sc_phase_transition(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    PFields F = B.P(), X = B.Pnext();
    SC_BATCHED(k_transition)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, &B.ctr->nActive, &B.ctr->step, F.pos, F.rot,
                                                           F.info, F.state, X.state, F.nb, X.nb, F.bonds, X.bonds,
                                                           F.lscs, F.spoly);
    B.cp[FP_STATE] ^= 1;
    B.cp[FP_NB] ^= 1;
    B.cp[FP_BONDS] ^= 1;
    (*c.launches)++;
}

void sc_phase_polymerize(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    PFields F = B.P();
    const int nb = nblocks(c.P.N);
    k_poly_count<<<nb, SC_THREADS, 0, c.st>>>(c.P, F, B.ctr, B.polyBlk);
    k_poly_offsets<<<1, SC_POLY_SCAN_THREADS, 0, c.st>>>(B.polyBlk, B.polyBlk + nb, nb, B.ctr);
    k_poly_plan<<<nb, SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, F, B.ctr, B.polyBlk + nb, B.polyList, B.polyRank,
                                             B.polyPmi, B.polyClaim);
    k_poly_apply<<<nb, SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, F, B.ctr, B.polyList, B.polyRank, B.polyPmi,
                                              B.polyClaim);
    k_poly_finish<<<1, 32, 0, c.st>>>(c.P, B.cellStartP, F, B.ctr, B.polyList, B.polyRank);
    (*c.launches) += 5;
}

void sc_phase_propagate_state(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.N <= 0) return;
    PFields F = B.P(), X = B.Pnext();
    SC_BATCHED(k_propagate_state)<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(
        c.P, B.cellStartP, &B.ctr->nActive, F.pos, F.info, F.state, X.state, F.lscs, X.lscs, F.nb, F.bonds);
    B.cp[FP_STATE] ^= 1;
    B.cp[FP_LSCS] ^= 1;
    (*c.launches)++;
}

void sc_phase_diffuse(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.Nm <= 0) return;
    MFields M = B.M(), X = B.Mnext();
    if (!B.validD) {
        // the build scratch follows the list in the same buffer
        cudaMemsetAsync(&B.ctr->ovfD, 0, sizeof(int), c.st);
        SC_BATCHED(k_build_d)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, B.cellStartM, &B.ctr->nActiveM, M.pos, M.info,
                                                             B.listD, B.listD + sc_list_words(SC_LIST_D, c.P.Nm),
                                                             B.cntD, B.permD, c.P.Nm, B.ovfD, &B.ctr->ovfD);
        cudaMemsetAsync(&B.ctr->poolOvfD, 0, sizeof(B.ctr->poolOvfD), c.st);
        SC_BATCHED(k_build_d_ovf)<<<std::min(nblocks(c.P.Nm), c.gridCap / 4), SC_THREADS, 0, c.st>>>(
            c.P, B.cellStartM, M.pos, M.info, B.ovfD, &B.ctr->ovfD, B.cntD, B.permD, B.ovfOffD, B.ovfPoolD,
            (long long)B.ovfPoolCapD, &B.ctr->poolOvfD);
        (*c.launches) += 2;
        B.validD = true;
    }
    PairList<SC_LIST_D> L;
    L.list = B.listD;
    L.cnt = B.cntD;
    L.cap = c.P.Nm;
    L.perm = B.permD;
    // the positions of the overflow pool run beside the others (on a side
    // stream when there is one): they write other items and read what the
    // others read
    const bool fork = c.side[0] != nullptr;
    cudaStream_t ps = fork ? c.side[0] : c.st;
    if (fork) {
        cudaEventRecord(c.fork, c.st);
        cudaStreamWaitEvent(ps, c.fork, 0);
    }
    const int pg = std::min(nblocks(c.P.Nm), c.gridCap);
    switch (c.P.SP) {
        case 4:
            k_diffuse_pool<4><<<pg, SC_THREADS, 0, ps>>>(c.P, M.info, L, B.ovfD, &B.ctr->ovfD, B.ovfOffD, B.ovfPoolD,
                                                         M.met, X.met);
            break;
        case 8:
            k_diffuse_pool<8><<<pg, SC_THREADS, 0, ps>>>(c.P, M.info, L, B.ovfD, &B.ctr->ovfD, B.ovfOffD, B.ovfPoolD,
                                                         M.met, X.met);
            break;
        default:
            k_diffuse_pool<12><<<pg, SC_THREADS, 0, ps>>>(c.P, M.info, L, B.ovfD, &B.ctr->ovfD, B.ovfOffD,
                                                          B.ovfPoolD, M.met, X.met);
    }
    (*c.launches)++;
    switch (c.P.SP) {
        case 4:
            (c.P.nRep > 1 ? k_diffuse<4, true> : k_diffuse<4, false>)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, B.cellStartM, &B.ctr->nActiveM, M.pos, M.info,
                                                                   L, M.met, X.met, B.ovfOffD, B.ovfPoolD);
            break;
        case 8:
            (c.P.nRep > 1 ? k_diffuse<8, true> : k_diffuse<8, false>)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, B.cellStartM, &B.ctr->nActiveM, M.pos, M.info,
                                                                   L, M.met, X.met, B.ovfOffD, B.ovfPoolD);
            break;
        default:
            (c.P.nRep > 1 ? k_diffuse<12, true> : k_diffuse<12, false>)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, B.cellStartM, &B.ctr->nActiveM, M.pos,
                                                                    M.info, L, M.met, X.met, B.ovfOffD, B.ovfPoolD);
            break;
    }
    if (fork) {
        cudaEventRecord(c.join[0], ps);
        cudaStreamWaitEvent(c.st, c.join[0], 0);
    }
    B.cm[FM_MET] ^= 1;
    (*c.launches)++;
}

void sc_phase_remove_interfering(ScLaunchCtx &c) {
    ScBuffers &B = *c.B;
    if (c.P.Nm <= 0) return;
    MFields M = B.M();
    PFields F = B.P();
    SC_BATCHED(k_remove_interfering)<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(c.P, B.cellStartP, &B.ctr->nActiveM, M.pos, M.info,
                                                                    F.pos, F.info);
    (*c.launches)++;
}

void sc_phase_reduce(ScLaunchCtx &c, int slot) {
    ScBuffers &B = *c.B;
    if (c.P.N > 0) {
        k_reduce_particles<<<nblocks(c.P.N), SC_THREADS, 0, c.st>>>(&B.ctr->nActive, c.P.N, B.P(),
                                                                     slot ? B.redP2 : B.redP);
        (*c.launches)++;
    }
    if (c.P.Nm > 0) {
        k_reduce_metabolic<<<nblocks(c.P.Nm), SC_THREADS, 0, c.st>>>(&B.ctr->nActiveM, c.P.Nm, c.P.SP / 4, B.M(),
                                                                      slot ? B.redM2 : B.redM);
        (*c.launches)++;
    }
}

// sc_launch.h -- buffers of one sim on the device and the launchers of its
// kernels (host side of the .cu files).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sc_dev.cuh"

struct PFields {
    float4 *pos, *vel, *rot, *angvel, *posnoise, *angnoise, *dbg;
    int4 *info;   // id, type, flags, hydrophobic
    int *state, *lscs, *spoly, *nb, *bonds;
};
struct MFields {
    float4 *pos, *vel, *rot, *angvel, *posnoise, *angnoise, *dbg;
    int4 *info;
    int *state;
    float4 *met;  // SP floats per item
    int *orig;
};

// Particle / metabolic field indices for the current-buffer table.
enum { FP_POS, FP_VEL, FP_ROT, FP_ANGVEL, FP_POSNOISE, FP_ANGNOISE, FP_DBG, FP_INFO, FP_STATE, FP_LSCS, FP_SPOLY,
       FP_NB, FP_BONDS, FP_COUNT };
enum { FM_POS, FM_VEL, FM_ROT, FM_ANGVEL, FM_POSNOISE, FM_ANGNOISE, FM_DBG, FM_INFO, FM_STATE, FM_MET, FM_ORIG,
       FM_COUNT };

struct ScBuffers {
    PFields p[2];
    MFields m[2];
    int cp[FP_COUNT];   // current buffer of each particle field
    int cm[FM_COUNT];   // current buffer of each metabolic field
    // metabolic fields no step kernel touches, in load order (indexed by orig)
    int *mcLscs, *mcSpoly, *mcNb, *mcBonds;
    // Loads whose metabolic records all hold no interactions and one value of
    // each of the other two fields keep those two values instead (mcUniform;
    // the four arrays above are then unallocated until a load needs them).
    bool mcUniform;
    int mcLscs0, mcSpoly0;
    int *mcFlag;   // device word of k_mc_scan
    // binning: keys / slot values ping-pong per item set, the buffer of the
    // last pass holding the sorted keys and the permutation
    uint32_t *keysP[2], *valsP[2], *keysM[2], *valsM[2], *hist, *lookback;
    int sortCurP, sortCurM;
    uint32_t *cellStartP, *cellStartM;
    // pair lists (sc_dev.cuh) and whether each matches the current state
    uint32_t *listPP, *listM, *listLM, *listD;
    int *cntPP, *cntM, *cntLM, *cntD;
    int *classPP;  // SC_RELAX_CLASSES segments of N item indices
    // Bond matches of the particle list: per bonded item, up to
    // SC_MAX_ACTIVE_INTERACTIONS entries (neighbour | bond slot << 29), in
    // list order then bond-slot order, and their count (k_build_pp).
    uint32_t *matchPP;
    int *matchN;
    int *permM, *permLM, *permD;  // count-ordered list position -> item
    uint32_t *scratchLM;          // build scratch of the LM list (aliases listD when it fits)
    int *ovfPP, *ovfM;            // overflowed items
    // The metabolic items whose list overflowed keep their full pair list in
    // a second pool (16-byte entries as the main one, an item's entries
    // contiguous): per overflow slot its pair count and first entry (-1: no
    // room, the item scans its neighbourhood)
    int *ovfNM;
    long long *ovfOffM;
    uint4 *ovfPoolM;
    size_t ovfPoolCapM;
    // the same for the diffusion lists: the overflowed list positions, the
    // first entry of each one's region by position (-1: it scans), neighbour
    // slots as entries
    int *ovfD;
    long long *ovfOffD;
    uint32_t *ovfPoolD;
    size_t ovfPoolCapD;
    long long *warpOffM;          // metabolic pair pool: first entry of every warp's region
    int *workP;                   // particle work list (the items complexify scans)
    unsigned long long *claimP;   // pair-claim keys, one per particle slot (sc_config.pair_claim)
    size_t poolCapM;              // entries the metabolic pair pool (listM) holds
    int poolEntryWords;           // 4-byte words per metabolic pool entry: 1 (lean) or 4 (with geometry)
    long long *warpOffLM;         // lipid-metabolic pair pool: the same
    uint8_t *lipidP;              // per sorted particle slot: active lipid (after each particle sort)
    bool validPP, validM, validLM, validD;
    void invalidateLists() { validPP = validM = validLM = validD = false; }
    // polymerisation list
    // polymerize: the scheduled items in index order, per slot the rank of
    // its new monomer and its previous monomer, per item a claim count, per
    // block of items its two counts and their offsets
    int *polyList, *polyRank, *polyPmi, *polyClaim;
    int2 *polyBlk;
    ScCounters *ctr;
    // frames
    sc_reduced_particle *redP, *redP2;                // frame staging, two slots
    sc_reduced_metabolic_particle *redM, *redM2;

    // current view of every particle / metabolic field
    PFields P() const {
        PFields f;
        f.pos = p[cp[FP_POS]].pos; f.vel = p[cp[FP_VEL]].vel; f.rot = p[cp[FP_ROT]].rot;
        f.angvel = p[cp[FP_ANGVEL]].angvel; f.posnoise = p[cp[FP_POSNOISE]].posnoise;
        f.angnoise = p[cp[FP_ANGNOISE]].angnoise; f.dbg = p[cp[FP_DBG]].dbg; f.info = p[cp[FP_INFO]].info;
        f.state = p[cp[FP_STATE]].state; f.lscs = p[cp[FP_LSCS]].lscs; f.spoly = p[cp[FP_SPOLY]].spoly;
        f.nb = p[cp[FP_NB]].nb; f.bonds = p[cp[FP_BONDS]].bonds;
        return f;
    }
    PFields Pnext() const {
        PFields f;
        f.pos = p[1 - cp[FP_POS]].pos; f.vel = p[1 - cp[FP_VEL]].vel; f.rot = p[1 - cp[FP_ROT]].rot;
        f.angvel = p[1 - cp[FP_ANGVEL]].angvel; f.posnoise = p[1 - cp[FP_POSNOISE]].posnoise;
        f.angnoise = p[1 - cp[FP_ANGNOISE]].angnoise; f.dbg = p[1 - cp[FP_DBG]].dbg;
        f.info = p[1 - cp[FP_INFO]].info; f.state = p[1 - cp[FP_STATE]].state;
        f.lscs = p[1 - cp[FP_LSCS]].lscs; f.spoly = p[1 - cp[FP_SPOLY]].spoly; f.nb = p[1 - cp[FP_NB]].nb;
        f.bonds = p[1 - cp[FP_BONDS]].bonds;
        return f;
    }
    MFields M() const {
        MFields f;
        f.pos = m[cm[FM_POS]].pos; f.vel = m[cm[FM_VEL]].vel; f.rot = m[cm[FM_ROT]].rot;
        f.angvel = m[cm[FM_ANGVEL]].angvel; f.posnoise = m[cm[FM_POSNOISE]].posnoise;
        f.angnoise = m[cm[FM_ANGNOISE]].angnoise; f.dbg = m[cm[FM_DBG]].dbg; f.info = m[cm[FM_INFO]].info;
        f.state = m[cm[FM_STATE]].state; f.met = m[cm[FM_MET]].met; f.orig = m[cm[FM_ORIG]].orig;
        return f;
    }
    MFields Mnext() const {
        MFields f;
        f.pos = m[1 - cm[FM_POS]].pos; f.vel = m[1 - cm[FM_VEL]].vel; f.rot = m[1 - cm[FM_ROT]].rot;
        f.angvel = m[1 - cm[FM_ANGVEL]].angvel; f.posnoise = m[1 - cm[FM_POSNOISE]].posnoise;
        f.angnoise = m[1 - cm[FM_ANGNOISE]].angnoise; f.dbg = m[1 - cm[FM_DBG]].dbg;
        f.info = m[1 - cm[FM_INFO]].info; f.state = m[1 - cm[FM_STATE]].state; f.met = m[1 - cm[FM_MET]].met;
        f.orig = m[1 - cm[FM_ORIG]].orig;
        return f;
    }
    void flipAllP() { for (int k = 0; k < FP_COUNT; k++) cp[k] ^= 1; }

    // Metabolic fields no step kernel double-buffers (every one but vel and
    // met) have one buffer each plus one spare per element size.  A sort
    // gathers them one field at a time into the spare, which then takes the
    // field's place: chain k of mChain4 / mChain1 (k >= 1) is field k - 1's
    // buffer at parity 0 and field k's at parity 1, chain entry 0 the spare
    // at parity 0; sorts alternate the parity, so buffers return every two.
    static constexpr int kM4 = 7, kM1 = 2;  // pos rot angvel posnoise angnoise dbg info | state orig
    float4 *mChain4[kM4 + 1];
    int *mChain1[kM1 + 1];
    int mParity;
    float4 **mField4(int k) {
        switch (k) {
            case 0: return &m[0].pos;
            case 1: return &m[0].rot;
            case 2: return &m[0].angvel;
            case 3: return &m[0].posnoise;
            case 4: return &m[0].angnoise;
            case 5: return &m[0].dbg;
            default: return reinterpret_cast<float4 **>(&m[0].info);
        }
    }
    int **mField1(int k) { return k == 0 ? &m[0].state : &m[0].orig; }
    void setMParity(int par) {
        mParity = par;
        for (int k = 0; k < kM4; k++) *mField4(k) = mChain4[k + 1 - par];
        for (int k = 0; k < kM1; k++) *mField1(k) = mChain1[k + 1 - par];
    }
    float4 *mSpare4() const { return mChain4[mParity ? kM4 : 0]; }
    int *mSpare1() const { return mChain1[mParity ? kM1 : 0]; }
};

// sc_grid.cu
int sc_sort_passes(int bits);
int sc_sort_passes_for(const ScParams &P);  // passes over P's key bits
size_t sc_sort_lookback_words(int cap);
int sc_launch_sort(cudaStream_t st, const float4 *pos, const int4 *info, int n, const ScParams &P, uint32_t *keys[2],
                   uint32_t *vals[2], uint32_t *hist, uint32_t *lookback, ScCounters *ctr, long long *launches);
void sc_launch_cell_start(cudaStream_t st, const uint32_t *keys, int n, uint32_t cells, uint32_t *cellStart,
                          long long *launches);
void sc_launch_gather_particles(cudaStream_t st, const uint32_t *perm, int n, const PFields &src, const PFields &dst,
                                long long *launches);
void sc_launch_gather_metabolic(cudaStream_t st, const uint32_t *perm, int n, int sp4, ScBuffers &B,
                                long long *launches);

// sc_observe.cu: FP64 observables.  The observe launcher reduces one item set
// into out[sc_observe_cols()] through a partials table of
// sc_observe_rows() x sc_observe_cols() doubles (columns: MSD sum, MSD
// items, |v|^2 sum, active items, bond slots, then one per species).
int sc_observe_cols();
int sc_observe_rows();
void sc_launch_mark(cudaStream_t st, const int *nActive, const float4 *pos, const int4 *info, float4 *mark,
                    int markCap);
void sc_launch_observe(cudaStream_t st, const int *nActive, const float4 *pos, const float4 *vel, const int4 *info,
                       const int *nb, const float *met, int sp, int S, const float4 *mark, int markCap, double box,
                       int periodic, double *partials, double *out);
void sc_launch_pair_histogram(cudaStream_t st, const ScParams &P, const uint32_t *cellStart, const int *nActive,
                              const float4 *pos, const int4 *info, int typeA, int typeB, double rMax, int nBins,
                              unsigned long long *counts, int gridCap);

// sc_step.cu: one launcher per reference phase (include/spatialcell.h, sc_phase)
struct ScLaunchCtx {
    cudaStream_t st;
    ScParams P;
    ScBuffers *B;
    long long *launches;
    int gridCap;  // blocks of SC_THREADS resident on the whole device (grid-stride kernels)
    // Two more streams for independent kernels of one phase: forked from st
    // at `fork`, joined back into st through join[0..1] before the phase ends
    // (null: everything runs on st).
    cudaStream_t side[2];
    cudaEvent_t fork, join[2];
};
void sc_phase_move_brownian(ScLaunchCtx &c, bool metabolic);
void sc_phase_coordinate_noise(ScLaunchCtx &c, float frac);
void sc_phase_apply_noise(ScLaunchCtx &c);
void sc_phase_relax(ScLaunchCtx &c);
void sc_phase_relax_metab(ScLaunchCtx &c);
void sc_phase_build_m(ScLaunchCtx &c);  // the relaxation's metabolic pair list alone
void sc_phase_relax_partners(ScLaunchCtx &c);
void sc_phase_build_lm(ScLaunchCtx &c);  // relax_partners' lipid-metabolic pair list alone
void sc_phase_apply_velocities(ScLaunchCtx &c);
// prep: the complexify of the start-up sequence (main.cu:324-336, step
// argument -1); otherwise the step's own, at the device step counter
void sc_phase_complexify(ScLaunchCtx &c, bool prep);
void sc_phase_transition(ScLaunchCtx &c);
void sc_phase_polymerize(ScLaunchCtx &c);
void sc_phase_propagate_state(ScLaunchCtx &c);
void sc_phase_diffuse(ScLaunchCtx &c);
void sc_phase_remove_interfering(ScLaunchCtx &c);
void sc_phase_reduce(ScLaunchCtx &c, int slot);
void sc_tile_init();
size_t sc_tile_bytes(int capM, int capP, int perSlot);

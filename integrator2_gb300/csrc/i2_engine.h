// i2_engine.h -- internal interfaces between the C-ABI layer (i2_capi.cu) and the kernels.
#pragma once

#include <algorithm>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "i2_device.cuh"
#include "i2_device_f32.cuh"
#include "i2_rules.cuh"

namespace i2 {

// depth cap of the adaptive potential rule (sub-cell paths of up to 24 bits)
constexpr int kHardMaxDepth = 12;
// a needle cell has a corner below 5 degrees: the mixed form computes the pairs that hold one (K_j
// only, for the disjoint class) in FP64; cos 5 degrees, compared with the panel's largest corner cosine
constexpr double kNeedleCos = 0.99619469809174553;
// the mixed form also recomputes in FP64 the adjacent pairs whose closed-form part exceeds the
// complete J by this factor: their FP32 quadrature part is as large, and its rounding (0.5-1.3e-7
// of J per unit of the ratio) is amplified by it.  48 bounds that amplification for 0.01 % of the
// common-vertex pairs of the 20,480-triangle jittered sphere (15 pairs; their ratios reach 355);
// 8 took 457 pairs there, cost 7 % of the step and left most of the FP32 tail, which is rounding
// on moderately conditioned pairs
constexpr double kFixRatio = 48.0;
// the common-edge closed form divides by 1 - c^2 (c = cos of the angle between the shared edge's
// neighbouring edges of the two cells, across the fold): a nearly coplanar pair whose cells have
// nearly equal angles there, short of the coplanar branch, cancels by that factor; the mixed form
// evaluates such pairs' closed form in FP64 below this value.  Double-float lost about
// 2e-15 / (1 - c^2) of J (4e-5 at 1 - c^2 = 5e-11 on the reference's Fish example), so 1e-7 keeps
// it near 2e-8; 1e-5 sent 3.4 % of a jittered torus grid's common-edge pairs there, and the FP64
// lanes slowed two thirds of its warps
constexpr double kEdgeClosedFormC2 = 1e-7;
// floats per adjacent pair in ClassArgs::ctx_e (mixed precision): the common-vertex asymptote's
// directions, or the common-edge pair's shared-edge term and shared-edge frame
constexpr int kPairCtxFloats = 20;
// ClassArgs::cnt, 16 ints per class run: [L] pairs still active after level L (L = 1..7),
// then the counters below
constexpr int kCntHard = 8;       // pairs handed to the adaptive potential rule
constexpr int kCntOverflow = 9;   // adaptive-rule cells kept because a depth's list was full
constexpr int kCntTier2 = 10;     // pairs the tier-1 potential check rejected
constexpr int kCntFixup = 11;     // pairs recomputed in FP64 by the mixed form (needle cells, kFixRatio)
constexpr int kCntTier2b = 12;    // pairs that reached tier 2b
constexpr int kCntFixDeep = 13;   // FP64 fix-up pairs whose deeper levels were spread over the GPU
// FP64 fix-up pairs per class run whose levels 4..5 can be spread over the GPU (820 KB of chunk
// sums); further deep pairs stay with their own block
constexpr int kFixDeepCap = 1024;
constexpr int kFixDeepSlots = 20;  // chunks of 64 sub-cells in levels 4 and 5
// refinement / error-control modes
enum { kFixed = 0, kAdaptiveCompat = 1, kAdaptiveRelative = 2 };

struct RunConfig {
    int mode = kFixed;
    int level = 0;        // fixed refinement level
    int max_level = kMaxLevel;
    double tol = 1e-6;    // relative tolerance of the adaptive relative mode
    int self_sign = 0;    // self-class normal convention
    double hard_tol = 1e-8;  // relative tolerance of the adaptive potential of hard adjacent pairs (0: off)
    bool potential = true;   // false: J only, as the reference computes (adjacent pairs' P is not computed)
};

// doubles of one hard pair's cached set-up (PotPairCtx in i2_kernels_fp64.cu, 54 doubles;
// PotPairCtxD in i2_kernels_df.cu, 55)
constexpr int kPotCtxDoubles = 56;

// one cell of the breadth-first adaptive potential rule of hard adjacent pairs
struct PotCellItem {
    unsigned long long path;  // base-4 digits of the sub-cell of K_i, first split most significant
    double val;               // the cell's integral by its own rule
    int h;                    // slot in the hard-pair list (-1: empty slot left by a full list)
    int corner;               // slot of the shared vertex in this cell, -1 if none
};
static_assert(sizeof(PotCellItem) == 24, "queue item is 24 bytes");

// everything a class's kernel chain reads and writes (device pointers)
struct ClassArgs {
    int n = 0;
    const int2 *pairs = nullptr;  // (i, j) per pair
    const int3 *cells = nullptr;
    const Panel *panels = nullptr;
    const PanelF *panels_f = nullptr;         // FP32 panel records (mixed precision)
    float *ctx_e = nullptr;                   // per-pair constants of the adjacent classes (mixed precision),
                                              // kPairCtxFloats floats per pair
    // per-pair state: regular-part sums (Psi, Theta, potential)
    double *cur = nullptr, *fin_a = nullptr, *fin_b = nullptr;
    int *stop = nullptr;
    int *act_a = nullptr, *act_b = nullptr;  // active-list ping-pong buffers
    int *act_in = nullptr, *act_out = nullptr;
    int *cnt = nullptr;                       // cnt[level] = pairs still active after level
    int *cnt_in = nullptr, *cnt_out = nullptr;
    int *maxlev = nullptr;
    double *sing = nullptr;                   // closed-form singular part (Psi, Theta)
    double *padj = nullptr;                   // potential of adjacent pairs
    int *hard_list = nullptr, *hard_cnt = nullptr;  // adjacent pairs whose potential is refined adaptively
    int *tier2_list = nullptr, *tier2_cnt = nullptr;  // pairs re-integrated with the higher-order Duffy rule
    int *tier2b_list = nullptr;               // pairs tier 2 rejected (count in cnt[kCntTier2b])
    // FP64 fix-up pairs whose levels 4..5 run spread over the GPU: the pairs, their level-3 sums
    // (5 doubles each), 20 chunk sums each (5 doubles), at most fix_cap pairs
    int *fix_deep = nullptr;
    double *fix_base = nullptr, *fix_part = nullptr;
    int fix_cap = 0;
    int *hard_overflow = nullptr;             // cells accepted early because a depth's list was full (diagnostic)
    PotCellItem *pot_q_a = nullptr, *pot_q_b = nullptr;  // adaptive potential: cell lists of two successive depths
    int pot_qcap = 0;                         // capacity of each list (>= 4 x hard pairs)
    int *pot_qcnt = nullptr;                  // cells per depth (kHardMaxDepth + 2 ints)
    long long *pot_fx = nullptr;              // per hard pair: accepted sums in 64-bit fixed point
    // caches of the adaptive potential, bit-identical to recomputing (entries past a cap are
    // recomputed): per hard pair its FP64 set-up (kPotCtxDoubles doubles, written by the seed),
    // and per splitting cell its triangle (9 doubles at the children's slot / 4 in the next
    // depth's list; two ping-pong arrays like the cell lists)
    double *pot_ctx = nullptr;
    int pot_ctx_cap = 0;
    double *pot_tri_a = nullptr, *pot_tri_b = nullptr;
    int pot_tri_cap = 0;
    double tier_tol = 1e-7;                   // main/check (and main/higher-order) rule agreement bar
    int pot_off = 0;                          // 1: J only; adjacent pairs' potential is not computed (P reads NaN)
    double top_tol = 1e-8;                    // 16 x 16 / 24 x 24 agreement bar (tier 2b)
    // outputs
    double *raw4 = nullptr, *J3 = nullptr, *P = nullptr;
    int *level_out = nullptr;
};

void launch_prepare_panels(int nc, const double *V, const int *C, Panel *out, cudaStream_t s);
void launch_prepare_panels_f32(int nc, const double *V, const int *C, PanelF *out, cudaStream_t s);
void launch_class_fp64(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks,
                       cudaStream_t s);
// a second stream and two events: work forked from a run's stream and joined back to it
struct SideStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};
void launch_class_mixed(int cls, const ClassArgs &A, const QuadTables &Q, const QuadTablesF &Qf, const RunConfig &cfg,
                        int persistent_blocks, cudaStream_t s, const SideStream &side);
// batched form: one segment = the pairs of one class of one mesh
struct BatchSeg {
    ClassArgs A;
    int cls;
};
// variant 0: registers unconstrained; 1: capped at 128 per thread (two 256-thread blocks per SM);
// the largest resident block count of the three class kernels
int batch_max_blocks_per_sm(int threads, int variant);
// bps: blocks per SM, capped at each class kernel's own maximum (0: the maximum); present[cls]:
// some segment holds pairs of class cls (0..2)
cudaError_t launch_batch_levels(const BatchSeg *segs, int nseg, const bool present[3], const QuadTablesF &Qf, const RunConfig &cfg,
                                int sms, int bps, int threads, int G_cap, int variant, cudaStream_t s);
// sizes the host knows about a batch (launch shapes of the batched stages)
struct BatchTotals {
    long long adjacent_pairs = 0;  // pairs of common-edge and common-vertex segments
    long long self_pairs = 0;
    long long fixup_pairs = 0;     // pairs the FP64 fix-up screens (segments with an active list)
    bool hard_lists = false;       // some adjacent segment has the potential's tier lists
    bool present[3] = {false, false, false};  // some segment holds pairs of class 0, 1, 2
};
// every segment's counter reset and the closed forms of its adjacent pairs: one launch
void launch_batch_singular(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTablesF &Qf, cudaStream_t s);
// tier 1 with the self pairs, tiers 2 / 2b, the adaptive potential and the adjacent pairs' P: one
// launch per stage for the whole batch (independent of the level sweep and the needle fix-up)
void launch_batch_potential(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTables &Q, const QuadTablesF &Qf,
                            const RunConfig &cfg, int persistent_blocks, cudaStream_t s);
// tier 2b and the adaptive potential of every segment's hard pairs (seed, depths, final sums),
// in double-float (i2_kernels_df.cu)
void launch_batch_pot_df(const BatchSeg *segs, int nseg, const QuadTables &Q, double tol, int persistent_blocks, cudaStream_t s);
// mixed form, one class: tier 2b and the adaptive potential in double-float
void launch_pot_tiers_hard_df(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s);
// the FP64 fix-up of needle pairs after the level sweep, for every segment
void launch_batch_fixup(const BatchSeg *segs, int nseg, const BatchTotals &tot, const QuadTables &Q, const RunConfig &cfg,
                        int persistent_blocks, cudaStream_t s);
// adjoint: dL/dV += gJ . dJ/dV + gP dP/dV over the pairs of one class (fp32: FP32 dual numbers)
void launch_adjoint(int cls, bool fp32, const int2 *pairs, int n, const int3 *cells, const double *V, const int *stop,
                    const int *maxlev, const RunConfig &cfg, double tier_tol, double top_tol, const double *gJ, const double *gP, double *gradV,
                    const QuadTables &Q, int persistent_blocks, cudaStream_t s);
// mixed form: FP64 recomputation of the pairs with a needle cell (corner below 5 degrees, kNeedleCos)
void launch_fp64_fixup(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s);
// blocks of `kernel` that are resident at once on the current device (occupancy x SMs): the grid
// of the FP64 warp-per-item passes, whose items go to the warps warp-major (warp_item_index), so
// that every SM gets the same share and no partial second wave runs on a few SMs
int resident_grid(const void *kernel, int threads, size_t smem);
// sets the thread's message returned by i2_last_error()
void set_last_error(const std::string &msg);
// kernels shared by both forms
void launch_finalize(int cls, const ClassArgs &A, int mode, cudaStream_t s);
void launch_self(const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, cudaStream_t s);
void launch_pot_hard(int cls, const ClassArgs &A, const QuadTables &Q, const RunConfig &cfg, int persistent_blocks, cudaStream_t s);

} // namespace i2

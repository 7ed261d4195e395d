// kmc.cuh -- launch wrappers of the KMC step kernels (kmc.cu).
#pragma once
#include <cuda_runtime.h>

#include "stz_internal.h"

namespace stz {

constexpr int kRateThreads = 256;
constexpr int kSptFp64 = 4;    // sites per thread of the FP64 rate kernels
constexpr int kGroup = 32;     // blocks per group in the two-level rate sums

// Rate kernel of the FP64 forms (ActEnergy + KMC rates + selection/commit in
// the last block). model: STZ_MODEL_REF2D or STZ_MODEL_GLOBAL3D.
void launch_rate_fp64(const KParams& kp, const Fields& f, cudaStream_t st);
// Mixed form: incremental stress update + rates + selection/commit.
// update_only: apply the pending transformation and uniform change, nothing else.
void launch_mixed(const KParams& kp, const Fields& f, int update_only, cudaStream_t st);
// One round of a batch: every replica's update/rate blocks in one grid, then
// one selection/commit block per replica.
// Kernels per thermal event of the mixed form: main pass, plane sums with the
// selection in their last block.
constexpr int kMixedLaunches = 2;
// Line-length classes of a batch: replicas with lines of 32, 64, 96 or 128 sites
// run the main pass specialised to that length, the rest the general pass.
// Their blocks occupy contiguous ranges of blk_rep, one launch per class,
// side by side on forked streams.
constexpr int kBatchClasses = 5;
constexpr int kBatchClassN2[kBatchClasses] = {32, 64, 96, 128, 0};
int batch_class(int n2);
struct BatchLaunch {
  int start[kBatchClasses] = {};   // first block of the class in blk_rep
  int count[kBatchClasses] = {};   // its blocks
  int max_n2[kBatchClasses] = {};  // its longest line (shared memory)
  cudaStream_t side[kBatchClasses] = {};
  cudaEvent_t fork = nullptr, join[kBatchClasses] = {};
};
void launch_mixed_batched(const BatchDesc* d, const int* blk_rep, const int* rep_first, const BatchLaunch& bl,
                          BatchStatus* status, int nrep, int max_n0, const ModeSet* shared, cudaStream_t st);
// Resident blocks per SM of the mixed-form kernel (occupancy query).
int mixed_blocks_per_sm(int n2);
// Dynamic shared memory of one mixed-form main block for lines of n2 sites.
size_t mixed_smem(int n2);
// the stored mode norms of the 2D model, after its mode increments were written
void launch_mode_norms(const KParams& kp, const Fields& f, cudaStream_t st);
// bounded-wait self-test kernel (one block); *kmax receives the kernels' limit
int wait_selftest(int tries, int* status_dev, int* kmax, cudaStream_t st);
// The two halves of launch_mixed: the grid-wide update/rate kernel and the
// one-block selection/commit kernel.
void launch_mixed_main(const KParams& kp, const Fields& f, int update_only, cudaStream_t st);
void launch_mixed_tail(const KParams& kp, const Fields& f, int update_only, cudaStream_t st);
// Athermal avalanche (evolution.c:47-100): mark sites, then commit in order.
void launch_athermal(const KParams& kp, const Fields& f, int mixed, cudaStream_t st);
// Bookkeeping after the solve of a step (loading, clock, print check) and
// after the optional print re-solve (stop checks, targets).
void launch_post_a(const KParams& kp, const Fields& f, cudaStream_t st);
void launch_post_b(const KParams& kp, const Fields& f, cudaStream_t st);
// FP64 incremental form: the thermal event's update of the field (two kernels,
// gated on the control block), and the mean strain of an FFT solve (gated as
// the solve)
void launch_incr64(const KParams& kp, const Fields& f, cudaStream_t st);
void launch_note_solve(const Fields& f, const int* gate, const double* ebar, cudaStream_t st);
// REF2D with crystal-like sites: restore the initial barriers when the step printed
void launch_q0_reset(const KParams& kp, const Fields& f, cudaStream_t st);
// Reset of the incremental state after a full re-solve (mixed form).
// kind 0: field solved with the current mean strain (print / athermal);
// kind 1: periodic re-solve with the applied mean strain (field unchanged).
void launch_mixed_after_resolve(const KParams& kp, const Fields& f, int kind, cudaStream_t st);
// Q of one mode at every site for the current field.
void launch_q_mode(const KParams& kp, const Fields& f, int mode, double* out, cudaStream_t st);
// Mixed-form helpers: deviatoric coordinates of an FP64 field, response table.
void launch_dev_from_sig(const KParams& kp, const double* sig, float* sdev, cudaStream_t st);
void launch_ktab_column(const KParams& kp, const double* sig, float* ktab, int b, cudaStream_t st);
void launch_fill_f32(const double* in, float* out, long long n, cudaStream_t st);
// Polarisation fixed point of a spatially varying medium (plain forms): the
// start (tau0, eeff from eps0 and the device mean strain ebar) and one update
// after a homogeneous solve of eigenstrain inh_last into sig; the update
// leaves kInhomBlocks partial sums of the squared change in inh_part.
constexpr int kInhomBlocks = 608;
void launch_inhom_init(const KParams& kp, const Fields& f, const double* ebar, cudaStream_t st);
void launch_inhom_update(const KParams& kp, const Fields& f, cudaStream_t st);
void launch_l2_flush(void* buf, size_t bytes, cudaStream_t st);
// One-warp kernel that keeps the stream busy for about ns nanoseconds, so the
// launches queued behind it start back to back (kernel timing).
void launch_hold(unsigned long long ns, cudaStream_t st);

}  // namespace stz

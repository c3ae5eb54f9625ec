/* CPU oracle for sequential-recombination jet clustering (TEST INFRASTRUCTURE).
 *
 * This is the checker, not the product: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg link it.  The product path is the CUDA
 * library under fastjet_gpu_gb300/csrc and never calls into this file.
 *
 * It restates, in plain C (FP64, no FMA contraction), the clustering the
 * reference backends implement: kt (p=1), Cambridge/Aachen (p=0) and anti-kt
 * (p=-1) with E-scheme recombination, distances
 *     d_iB = w_i,   d_ij = (min(w_i, w_j) * dR2_ij) * (1/R^2)
 * and the reference's rapidity/azimuth convention.  Selection is the canonical
 * rule shared with the CUDA kernels (nearest-neighbour table, lowest-label
 * tie-break); see fjg_oracle.c for the citations.
 */
#ifndef FJG_ORACLE_H
#define FJG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Algorithm codes: the reference's enum values (cluster.h:4), i.e. the exponent p. */
enum { FJO_KT = 1, FJO_CAM = 0, FJO_ANTIKT = -1 };

/* Methods: incremental nearest-neighbour update (O(N^2)) or a full
 * nearest-neighbour recomputation at every step (O(N^3), a cross-check). */
enum { FJO_NN_INCREMENTAL = 0, FJO_NN_RECOMPUTE = 1 };

/* OR into `method`: compute rapidity/azimuth/weights with the library's
 * integer kinematics (fastjet_gpu_gb300/csrc/fjg_kin.h) instead of the host
 * libm.  The default (libm) form is the one pinned to the reference outputs;
 * the portable form makes the oracle's arithmetic bit-identical to the CUDA
 * kernels', so tests can demand exact equality even for ties that hinge on
 * the last bit of log/atan2. */
enum { FJO_KIN_PORTABLE = 16 };

typedef struct {
  int32_t a;  /* label of the first pseudojet (the smaller label for a merge) */
  int32_t b;  /* label of the second pseudojet, or -1 when a is promoted to a jet */
  double d;   /* the winning distance d_ab or d_aB */
} fjo_step;

/* Per-particle derived kinematics, exactly as the reference computes them
 * (tri_matrix.cu:61-100): pt2, phi in [0, 2pi), rapidity, and the weight w
 * (kt: pt2, C/A: 1, anti-kt: 1/pt2 guarded at 1e-300). */
void fjo_kinematics(const double p4[4], int algo, double* pt2, double* phi, double* rap, double* w);

/* The library's integer log / atan2 / division (fjg_kin.h), for tests. */
double fjo_kin_log(double x);
double fjo_kin_atan2(double y, double x);
double fjo_kin_div(double a, double b);
float fjo_kin_f32(double x, int mode); /* mode 0: nearest, 1: toward -inf, 2: toward +inf */
void fjo_kin_kinematics(const double p4[4], int algo, double* rap, double* phi, double* w);

/* Cluster one event of n particles (p4: [n][4] px,py,pz,E).
 * Outputs (any may be NULL):
 *   history  [n]     one record per step, in step order
 *   jets     [n][4]  final inclusive jets in promotion order
 *   jet_label[n]     label (lowest constituent input index) of each jet
 *   owner    [n]     for each input particle, the index of its jet in jets[]
 *   n_jets           number of jets
 *   pair_evals       number of pair distances evaluated (algorithmic work count)
 * Returns 0 on success, -1 on invalid arguments or allocation failure. */
int fjo_cluster(const double* p4, int n, int algo, double R, int method, fjo_step* history, double* jets,
                int32_t* jet_label, int32_t* owner, int* n_jets, long long* pair_evals);

/* Cluster a CSR batch (offsets[n_events+1]) with `threads` POSIX threads, one
 * event per task (threads | FJO_KIN_PORTABLE << 16 selects the portable
 * kinematics).  Outputs are CSR-indexed by the same offsets: history[total],
 * jets[total][4], jet_label[total], owner[total]; n_jets[n_events].  Any output
 * may be NULL.  Returns 0 on success. */
int fjo_cluster_batch(const double* p4, const int64_t* offsets, int n_events, const int32_t* algo,
                      const double* R, int threads, fjo_step* history, double* jets, int32_t* jet_label,
                      int32_t* owner, int32_t* n_jets, long long* pair_evals);

#ifdef __cplusplus
}
#endif

#endif

/* CPU oracle for sequential-recombination jet clustering (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
 * this file.  It must be compiled with -ffp-contract=off so that every FP64
 * expression rounds exactly as written (the CUDA kernels use explicit
 * __dmul_rn/__dadd_rn for the same expressions).
 *
 * What it restates from the reference (fwyzard/fastjet_gpu):
 *   - kinematics  : tri_matrix.cu:61-100 (_set_jet: pt2, phi folded into
 *                   [0, 2pi), massive-safe rapidity with the MaxRap=1e5 branch
 *                   for E == |pz| and pt2 == 0), grid.cu:153-166 (weight per
 *                   algorithm), grid.cu:110 (safe_inverse: 1/pt2 guarded at
 *                   1e-300 -> 1e300);
 *   - distance    : tri_matrix.cu:102-109 (plain_distance: dphi folded at pi,
 *                   dphi^2 + drap^2), tri_matrix.cu:111-113 (yij_distance:
 *                   (min(w_i, w_j) * dR2) * one_over_r2, left to right),
 *                   one_over_r2 = 1./(r*r) in double (tri_matrix.cu:305);
 *   - beam distance d_iB = w_i (tri_matrix.cu:40-53, grid.cu:194-195);
 *   - recombination: E-scheme, component-wise sum (tri_matrix.cu:248-252);
 *   - promotion   : the pseudojet becomes a final jet (tri_matrix.cu:241-246).
 *
 * Selection rule (shared bit-for-bit with the CUDA kernels).  Every active
 * pseudojet s has a label (the lowest input index among its constituents) and
 * a geometric nearest neighbour nn(s) = argmin_t (dR2_st, label_t) over the
 * other active pseudojets.  Its candidate key is
 *     d_pair = (min(w_s, w_nn) * dR2_s,nn) * one_over_r2,
 *     key_s  = d_pair < w_s ? d_pair (merge with nn) : w_s (promote s),
 * and each step takes argmin_s (key_s, label_s).  For the pair (a, b) that
 * minimises d over all pairs with w_a <= w_b, a's geometric neighbour c has
 * dR2_ac <= dR2_ab and min(w_a, w_c) <= w_a; FP64 rounding is monotone, so the
 * computed d_ac <= d_ab.  The selected value therefore equals the reference's
 * all-pairs minimum (tri_matrix.cu:161-257); only exact ties can pick a
 * different candidate, and the reference itself resolves those differently in
 * each backend (CUB lane order in tri_matrix/n_array, atomicCAS slot order in
 * grid).  The incremental update after a merge follows the nearest-neighbour
 * bookkeeping of the generalised-kt "N2Plain" strategy (Cacciari & Salam,
 * Phys. Lett. B 641 (2006) 57): only pseudojets whose neighbour was one of
 * the merged pair are rescanned, every other one is compared with the new jet.
 */
#include "fjg_oracle.h"

#include <math.h>

#include "fjg_kin.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static const double kPi = 3.141592653589793238462643383279502884197;
static const double kTwoPi = 6.283185307179586476925286766559005768394;
static const double kMaxRap = 1e5;

void fjo_kinematics(const double p4[4], int algo, double* pt2_out, double* phi_out, double* rap_out,
                    double* w_out) {
  const double px = p4[0], py = p4[1], pz = p4[2], E = p4[3];
  const double pt2 = px * px + py * py;
  double phi = (pt2 == 0.0) ? 0.0 : atan2(py, px);
  if (phi < 0.0) phi += kTwoPi;
  if (phi >= kTwoPi) phi -= kTwoPi;
  double rap;
  if (E == fabs(pz) && pt2 == 0.0) {
    const double max_rap_here = kMaxRap + fabs(pz);
    rap = (pz >= 0.0) ? max_rap_here : -max_rap_here;
  } else {
    double m2 = (E + pz) * (E - pz) - pt2;
    if (m2 < 0.0) m2 = 0.0;
    const double e_plus_pz = E + fabs(pz);
    rap = 0.5 * log((pt2 + m2) / (e_plus_pz * e_plus_pz));
    if (pz > 0.0) rap = -rap;
  }
  double w;
  if (algo == FJO_KT)
    w = pt2;
  else if (algo == FJO_CAM)
    w = 1.0;
  else
    w = (pt2 > 1e-300) ? 1.0 / pt2 : 1e300;
  if (pt2_out) *pt2_out = pt2;
  if (phi_out) *phi_out = phi;
  if (rap_out) *rap_out = rap;
  if (w_out) *w_out = w;
}

/* (d, l) ranks before (bd, bl): smaller distance, then smaller label */
static inline int closer(double d, int32_t l, double bd, int32_t bl) { return d < bd || (d == bd && l < bl); }

double fjo_kin_log(double x) { return fjk_log(x); }
double fjo_kin_atan2(double y, double x) { return fjk_atan2(y, x); }
double fjo_kin_div(double a, double b) { return fjk_div_rn(a, b); }
float fjo_kin_f32(double x, int mode) { return fjk_to_f32(x, mode); }
void fjo_kin_kinematics(const double p4[4], int algo, double* rap, double* phi, double* w) {
  fjk_kinematics(p4[0], p4[1], p4[2], p4[3], algo, rap, phi, w);
}

/* rapidity, azimuth and weight in the selected form (libm or portable) */
static inline void kin(const double p[4], int algo, int portable, double* phi, double* rap, double* w) {
  if (portable)
    fjk_kinematics(p[0], p[1], p[2], p[3], algo, rap, phi, w);
  else
    fjo_kinematics(p, algo, NULL, phi, rap, w);
}

static inline double delta_r2(double rap1, double phi1, double rap2, double phi2) {
  double dphi = fabs(phi1 - phi2);
  if (dphi > kPi) dphi = kTwoPi - dphi;
  const double drap = rap1 - rap2;
  return dphi * dphi + drap * drap;
}

typedef struct {
  double p[4];
  double rap, phi, w;
  int32_t label;
  int32_t nn;     /* slot of the nearest neighbour, -1 if none */
  double nndist;  /* dR2 to nn, +inf if none */
  double key;     /* candidate distance */
  int is_pair;    /* key is d_pair (merge with nn) rather than w (promote) */
} oj;

static void set_key(oj* J, int s, double inv_r2) {
  oj* a = &J[s];
  if (a->nn < 0) {
    a->key = a->w;
    a->is_pair = 0;
    return;
  }
  const double wmin = a->w < J[a->nn].w ? a->w : J[a->nn].w;
  const double d = (wmin * a->nndist) * inv_r2;
  if (d < a->w) {
    a->key = d;
    a->is_pair = 1;
  } else {
    a->key = a->w;
    a->is_pair = 0;
  }
}

/* argmin over active t != s of (dR2_st, label_t) */
static void rescan(oj* J, const int* act, int n_act, int s, long long* evals) {
  int best = -1;
  double bd = INFINITY;
  int32_t bl = 0;
  for (int q = 0; q < n_act; ++q) {
    const int t = act[q];
    if (t == s) continue;
    const double d = delta_r2(J[s].rap, J[s].phi, J[t].rap, J[t].phi);
    ++*evals;
    if (best < 0 || closer(d, J[t].label, bd, bl)) {
      bd = d;
      best = t;
      bl = J[t].label;
    }
  }
  J[s].nn = best;
  J[s].nndist = bd;
}

static int find_root(int32_t* parent, int32_t x) {
  while (parent[x] != x) {
    parent[x] = parent[parent[x]];
    x = parent[x];
  }
  return x;
}

int fjo_cluster(const double* p4, int n, int algo, double R, int method, fjo_step* history, double* jets,
                int32_t* jet_label, int32_t* owner, int* n_jets_out, long long* pair_evals) {
  if (n < 0 || (n > 0 && !p4)) return -1;
  if (algo != FJO_KT && algo != FJO_CAM && algo != FJO_ANTIKT) return -1;
  const int portable = (method & FJO_KIN_PORTABLE) != 0;
  method &= ~FJO_KIN_PORTABLE;
  long long evals = 0;
  int n_jets = 0;
  if (n == 0) {
    if (n_jets_out) *n_jets_out = 0;
    if (pair_evals) *pair_evals = 0;
    return 0;
  }
  oj* J = (oj*)malloc(sizeof(oj) * (size_t)n);
  int* act = (int*)malloc(sizeof(int) * (size_t)n);
  int* pos = (int*)malloc(sizeof(int) * (size_t)n);
  int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int32_t* jet_of_root = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  if (!J || !act || !pos || !parent || !jet_of_root) {
    free(J); free(act); free(pos); free(parent); free(jet_of_root);
    return -1;
  }
  const double inv_r2 = 1.0 / (R * R);

  for (int s = 0; s < n; ++s) {
    memcpy(J[s].p, p4 + 4 * (size_t)s, sizeof(double) * 4);
    kin(J[s].p, algo, portable, &J[s].phi, &J[s].rap, &J[s].w);
    J[s].label = s;
    J[s].nn = -1;
    J[s].nndist = INFINITY;
    act[s] = s;
    pos[s] = s;
    parent[s] = s;
    jet_of_root[s] = -1;
  }
  int n_act = n;

  /* initial nearest neighbours: every pair once, both ends updated */
  for (int i = 0; i < n; ++i) {
    for (int j = i + 1; j < n; ++j) {
      const double d = delta_r2(J[i].rap, J[i].phi, J[j].rap, J[j].phi);
      ++evals;
      if (J[i].nn < 0 || closer(d, J[j].label, J[i].nndist, J[J[i].nn].label)) {
        J[i].nndist = d;
        J[i].nn = j;
      }
      if (J[j].nn < 0 || closer(d, J[i].label, J[j].nndist, J[J[j].nn].label)) {
        J[j].nndist = d;
        J[j].nn = i;
      }
    }
  }
  for (int s = 0; s < n; ++s) set_key(J, s, inv_r2);

  for (int step = 0; step < n; ++step) {
    if (method == FJO_NN_RECOMPUTE && step > 0) {
      for (int q = 0; q < n_act; ++q) {
        rescan(J, act, n_act, act[q], &evals);
        set_key(J, act[q], inv_r2);
      }
    }
    /* argmin over (key, label) */
    int best = act[0];
    for (int q = 1; q < n_act; ++q) {
      const int s = act[q];
      if (J[s].key < J[best].key || (J[s].key == J[best].key && J[s].label < J[best].label)) best = s;
    }
    const double dmin = J[best].key;

    if (!J[best].is_pair) {
      /* promote best to a final jet */
      if (history) {
        history[step].a = J[best].label;
        history[step].b = -1;
        history[step].d = dmin;
      }
      if (jets) memcpy(jets + 4 * (size_t)n_jets, J[best].p, sizeof(double) * 4);
      if (jet_label) jet_label[n_jets] = J[best].label;
      jet_of_root[find_root(parent, J[best].label)] = n_jets;
      ++n_jets;
      /* remove from the active list */
      const int q = pos[best];
      act[q] = act[n_act - 1];
      pos[act[q]] = q;
      --n_act;
      if (method == FJO_NN_INCREMENTAL) {
        for (int r = 0; r < n_act; ++r) {
          const int t = act[r];
          if (J[t].nn == best) {
            rescan(J, act, n_act, t, &evals);
            set_key(J, t, inv_r2);
          }
        }
      }
      continue;
    }

    /* merge best with its neighbour; the new jet takes the slot of best */
    const int i = best, j = J[best].nn;
    const int32_t li = J[i].label, lj = J[j].label;
    if (history) {
      history[step].a = li < lj ? li : lj;
      history[step].b = li < lj ? lj : li;
      history[step].d = dmin;
    }
    {
      const int32_t ri = find_root(parent, li), rj = find_root(parent, lj);
      if (ri < rj) parent[rj] = ri; else parent[ri] = rj;
    }
    for (int c = 0; c < 4; ++c) J[i].p[c] = J[i].p[c] + J[j].p[c];
    kin(J[i].p, algo, portable, &J[i].phi, &J[i].rap, &J[i].w);
    J[i].label = li < lj ? li : lj;
    {
      const int q = pos[j];
      act[q] = act[n_act - 1];
      pos[act[q]] = q;
      --n_act;
    }
    if (method == FJO_NN_INCREMENTAL) {
      /* new jet against everyone: its own neighbour, and neighbour updates of others */
      J[i].nn = -1;
      J[i].nndist = INFINITY;
      for (int r = 0; r < n_act; ++r) {
        const int t = act[r];
        if (t == i) continue;
        const double d = delta_r2(J[i].rap, J[i].phi, J[t].rap, J[t].phi);
        ++evals;
        if (J[i].nn < 0 || closer(d, J[t].label, J[i].nndist, J[J[i].nn].label)) {
          J[i].nndist = d;
          J[i].nn = t;
        }
        if (J[t].nn == i || J[t].nn == j) continue; /* rescanned below */
        if (J[t].nn < 0 || closer(d, J[i].label, J[t].nndist, J[J[t].nn].label)) {
          J[t].nndist = d;
          J[t].nn = i;
          set_key(J, t, inv_r2);
        }
      }
      set_key(J, i, inv_r2);
      for (int r = 0; r < n_act; ++r) {
        const int t = act[r];
        if (t == i) continue;
        if (J[t].nn == i || J[t].nn == j) {
          /* a neighbour that was i may still be the new jet i: rescan decides */
          rescan(J, act, n_act, t, &evals);
          set_key(J, t, inv_r2);
        }
      }
    }
  }

  if (owner) {
    for (int s = 0; s < n; ++s) owner[s] = jet_of_root[find_root(parent, s)];
  }
  if (n_jets_out) *n_jets_out = n_jets;
  if (pair_evals) *pair_evals = evals;
  free(J); free(act); free(pos); free(parent); free(jet_of_root);
  return 0;
}

/* ------------------------------------------------------------------ batch */

typedef struct {
  const double* p4;
  const int64_t* offsets;
  int n_events;
  const int32_t* algo;
  const double* R;
  fjo_step* history;
  double* jets;
  int32_t* jet_label;
  int32_t* owner;
  int32_t* n_jets;
  long long evals;
  int status;
  int kin_flag; /* FJO_KIN_PORTABLE or 0 */
  int* next;    /* shared work counter */
  pthread_mutex_t* mu;
} batch_task;

static void* batch_worker(void* arg) {
  batch_task* t = (batch_task*)arg;
  for (;;) {
    pthread_mutex_lock(t->mu);
    const int e = (*t->next)++;
    pthread_mutex_unlock(t->mu);
    if (e >= t->n_events) break;
    const int64_t o = t->offsets[e];
    const int n = (int)(t->offsets[e + 1] - o);
    int nj = 0;
    long long ev = 0;
    const int rc = fjo_cluster(t->p4 + 4 * o, n, t->algo[e], t->R[e], FJO_NN_INCREMENTAL | t->kin_flag,
                               t->history ? t->history + o : NULL, t->jets ? t->jets + 4 * o : NULL,
                               t->jet_label ? t->jet_label + o : NULL, t->owner ? t->owner + o : NULL, &nj, &ev);
    if (rc) t->status = rc;
    if (t->n_jets) t->n_jets[e] = nj;
    t->evals += ev;
  }
  return NULL;
}

int fjo_cluster_batch(const double* p4, const int64_t* offsets, int n_events, const int32_t* algo,
                      const double* R, int threads, fjo_step* history, double* jets, int32_t* jet_label,
                      int32_t* owner, int32_t* n_jets, long long* pair_evals) {
  const int kin_flag = (threads & FJO_KIN_PORTABLE << 16) ? FJO_KIN_PORTABLE : 0;
  threads &= 0xffff;
  if (n_events < 0 || !offsets || !algo || !R) return -1;
  if (threads < 1) threads = 1;
  if (threads > 1024) threads = 1024;
  int next = 0;
  pthread_mutex_t mu;
  pthread_mutex_init(&mu, NULL);
  batch_task* tasks = (batch_task*)calloc((size_t)threads, sizeof(batch_task));
  pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  if (!tasks || !tid) {
    free(tasks); free(tid);
    return -1;
  }
  for (int k = 0; k < threads; ++k) {
    batch_task* t = &tasks[k];
    t->p4 = p4; t->offsets = offsets; t->n_events = n_events; t->algo = algo; t->R = R;
    t->history = history; t->jets = jets; t->jet_label = jet_label; t->owner = owner; t->n_jets = n_jets;
    t->next = &next; t->mu = &mu; t->kin_flag = kin_flag;
  }
  int status = 0;
  for (int k = 1; k < threads; ++k)
    if (pthread_create(&tid[k], NULL, batch_worker, &tasks[k])) tasks[k].status = -2;
  batch_worker(&tasks[0]);
  long long evals = 0;
  for (int k = 0; k < threads; ++k) {
    if (k > 0 && tasks[k].status != -2) pthread_join(tid[k], NULL);
    if (tasks[k].status) status = tasks[k].status;
    evals += tasks[k].evals;
  }
  pthread_mutex_destroy(&mu);
  free(tasks); free(tid);
  if (pair_evals) *pair_evals = evals;
  return status;
}

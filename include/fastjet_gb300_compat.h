/* Drop-in replacement for the reference's plugin boundary (fwyzard/fastjet_gpu).
 *
 * Declares exactly the reference's types and entry point:
 *   PseudoJet.h:4-11  struct PseudoJet
 *   cluster.h:4       enum class Algorithm
 *   cluster.h:6       void cluster(PseudoJet *particles, int size, Algorithm algo, double r);
 * so the reference driver (main.cc) links against libfastjet_gb300.so unchanged
 * (C++ symbol _Z7clusterP9PseudoJeti9Algorithmd).
 *
 * Semantics: `particles` is a device buffer of `size` records, rewritten in
 * place on the legacy default stream of the current device; the call returns
 * once the results are in the buffer.  Final inclusive jets are the records
 * with isJet == true; each sits at the slot of its lowest-index constituent and
 * has index == that slot (the reference's grid backend also reports input
 * indices, grid.cu:575).  As in the reference (cudaCheck.h:32), a CUDA failure
 * prints a message to stderr and aborts the process.
 */
#ifndef FASTJET_GB300_COMPAT_H
#define FASTJET_GB300_COMPAT_H

#ifndef PseudoJet_h
#define PseudoJet_h
struct PseudoJet {
  int index;
  bool isJet;
  double px;
  double py;
  double pz;
  double E;
};
#endif

#ifndef cluster_h
#define cluster_h
enum class Algorithm { Kt = 1, CambridgeAachen = 0, AntiKt = -1 };

void cluster(PseudoJet *particles, int size, Algorithm algo, double r);
#endif

#endif /* FASTJET_GB300_COMPAT_H */

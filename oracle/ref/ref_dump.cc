// Parity harness for the reference backends (test infrastructure, not product).
//
// Links against exactly one of the reference's backend objects (tri_matrix.o,
// n_array.o or grid.o) and drives it through its public entry point
//   void cluster(PseudoJet *particles, int size, Algorithm algo, double r);
// (cluster.h:6), the way the reference driver does (main.cc:279-298): the event
// is copied to a device buffer, cluster() rewrites it in place, the buffer is
// copied back.  Every output slot is printed as
//   slot index isJet px py pz E        (momenta as C99 hex floats, exact)
// one line per slot, and each event ends with a line "end <N>".  Linked with
// the history-printing copy of a backend (stage_hist.py), the backend's own
// device printf adds one "H ..." line per clustering step before the slots; the
// printf FIFO is enlarged for that, as the reference driver does (main.cc:28),
// and stdout is flushed around every event so the lines stay in event order.
//
// usage: <backend>_dump (-kt|-antikt|-cam) R < events.txt
// Input: the reference's text format (px py pz E per line, events separated by
// blank or '#' lines; main.cc:34-70).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "PseudoJet.h"
#include "cluster.h"

static bool read_event(std::istream& in, std::vector<PseudoJet>& ev) {
  ev.clear();
  std::string line;
  bool started = false;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    double px, py, pz, E;
    if (ls >> px >> py >> pz >> E) {
      ev.push_back({(int)ev.size(), false, px, py, pz, E});
      started = true;
    } else if (started) {
      return true;  // blank or '#' line ends an event
    }
  }
  return started;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s (-kt|-antikt|-cam) R < events\n", argv[0]);
    return 2;
  }
  Algorithm algo;
  if (!std::strcmp(argv[1], "-kt")) algo = Algorithm::Kt;
  else if (!std::strcmp(argv[1], "-antikt")) algo = Algorithm::AntiKt;
  else if (!std::strcmp(argv[1], "-cam")) algo = Algorithm::CambridgeAachen;
  else { std::fprintf(stderr, "bad algorithm %s\n", argv[1]); return 2; }
  double r = std::strtod(argv[2], nullptr);
  // one step line takes ~200 bytes of the FIFO; room for events of ~1M particles
  if (cudaDeviceSetLimit(cudaLimitPrintfFifoSize, (size_t)256 << 20) != cudaSuccess) {
    std::fprintf(stderr, "cannot size the printf FIFO\n");
    return 1;
  }

  std::vector<PseudoJet> ev;
  while (read_event(std::cin, ev)) {
    PseudoJet* d = nullptr;
    size_t bytes = sizeof(PseudoJet) * ev.size();
    if (cudaMalloc(&d, bytes) != cudaSuccess) { std::fprintf(stderr, "cudaMalloc failed\n"); return 1; }
    cudaMemcpy(d, ev.data(), bytes, cudaMemcpyDefault);
    std::fflush(stdout);
    cluster(d, (int)ev.size(), algo, r);
    cudaMemcpy(ev.data(), d, bytes, cudaMemcpyDefault);
    cudaError_t err = cudaDeviceSynchronize();
    cudaFree(d);
    if (err != cudaSuccess) { std::fprintf(stderr, "CUDA error %s\n", cudaGetErrorString(err)); return 1; }
    for (size_t s = 0; s < ev.size(); ++s) {
      const PseudoJet& p = ev[s];
      std::printf("%zu %d %d %a %a %a %a\n", s, p.index, p.isJet ? 1 : 0, p.px, p.py, p.pz, p.E);
    }
    std::printf("end %zu\n", ev.size());
    std::fflush(stdout);
  }
  return 0;
}

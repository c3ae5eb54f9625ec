// fjg_cluster: command-line driver with the reference driver's interface
// (fwyzard/fastjet_gpu main.cc), running the GB300 clustering library.
//
// Same options (main.cc:129-257): --ptmin/-p, -r/-R, --repeat/-repeat,
// --sort/-s, --cartesian, --polar, --kt/-kt, --anti-kt/-antikt,
// --cambridge-aachen/-cam, --file/-f, --combine/-combine, --csv/-csv; same
// input stream (px py pz E per line, events separated by blank or '#' lines,
// main.cc:34-85); same per-event output (main.cc:269-367): particle count,
// jets above ptmin with the time of copy-in + clustering + copy-out, the jets
// sorted by decreasing pT in polar or cartesian form, and a summary or CSV
// line.  Added option (not in the reference): --batch clusters every event
// of the stream in one batched call (fjg_cluster_batch_host) and reports the
// time of that call.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fastjet_gb300.h"
#include "fastjet_gb300_compat.h"

namespace {

struct Options {
  double ptmin = 0.0;
  double r = 1.0;
  Algorithm algo = Algorithm::Kt;
  bool cartesian = false;
  long repetitions = 1;
  long combine = 1;
  std::string filename;
  bool csv = false;
  bool batch = false;
};

void check(cudaError_t err, const char* what) {
  if (err != cudaSuccess) {
    std::cerr << "\n" << what << ": " << cudaGetErrorName(err) << ": " << cudaGetErrorString(err) << std::endl;
    std::abort();
  }
}

// Parse argv like the reference: an option's value must parse completely at
// its start and be non-negative; a missing value or unknown option exits 1.
bool parse(int argc, const char* argv[], Options& o) {
  auto value = [&](int& i, const char* name) -> const char* {
    if (++i >= argc) {
      std::cerr << "Missing argument to option " << name << std::endl;
      return nullptr;
    }
    return argv[i];
  };
  auto bad = [](const char* name) {
    std::cerr << "Error while parsing argument to option " << name << std::endl;
    return false;
  };
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--ptmin" || a == "-p" || a == "-r" || a == "-R") {
      const char* v = value(i, argv[i]);
      if (!v) return false;
      char* stop;
      const double x = std::strtod(v, &stop);
      if (stop == v || !(x >= 0.)) return bad(argv[i - 1]);
      (a == "--ptmin" || a == "-p" ? o.ptmin : o.r) = x;
    } else if (a == "--repeat" || a == "-repeat" || a == "--combine" || a == "-combine") {
      const char* v = value(i, argv[i]);
      if (!v) return false;
      char* stop;
      const long x = std::strtol(v, &stop, 0);
      if (stop == v || x < 0) return bad(argv[i - 1]);
      (a == "--repeat" || a == "-repeat" ? o.repetitions : o.combine) = x;
    } else if (a == "--sort" || a == "-s") {
      // the reference always sorts (main.cc:122, 188-190)
    } else if (a == "--cartesian") {
      o.cartesian = true;
    } else if (a == "--polar") {
      o.cartesian = false;
    } else if (a == "--kt" || a == "-kt") {
      o.algo = Algorithm::Kt;
    } else if (a == "--anti-kt" || a == "-antikt") {
      o.algo = Algorithm::AntiKt;
    } else if (a == "--cambridge-aachen" || a == "-cam") {
      o.algo = Algorithm::CambridgeAachen;
    } else if (a == "--file" || a == "-f") {
      const char* v = value(i, argv[i]);
      if (!v) return false;
      o.filename = v;
    } else if (a == "--csv" || a == "-csv") {
      o.csv = true;
    } else if (a == "--batch") {
      o.batch = true;
    } else {
      std::cerr << "Unrecognized option " << argv[i] << std::endl;
      return false;
    }
  }
  return true;
}

// One event from the stream, appended to `particles` with running indices.
// Leading '#' and empty lines are skipped; the event ends at the first line
// that does not hold four numbers, which must be empty or start with '#'.  A
// final line without a newline is not read (std::getline reports eof).
bool read_event(std::istream& in, std::vector<PseudoJet>& particles) {
  in.clear();
  while (in.peek() == '#' || in.peek() == '\n') in.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  bool found = false;
  std::string line;
  while (std::getline(in, line).good()) {
    std::istringstream ls(line);
    double px, py, pz, E;
    ls >> px >> py >> pz >> E;
    if (ls.fail()) {
      if (!line.empty() && line[0] != '#') throw std::runtime_error("Error while parsing particles:\n" + line);
      break;
    }
    particles.push_back({static_cast<int>(particles.size()), false, px, py, pz, E});
    found = true;
  }
  return found;
}

long read_events(std::istream& in, std::vector<PseudoJet>& particles, long n) {
  particles.clear();
  long events = 0;
  while ((n == 0 || events < n) && read_event(in, particles)) ++events;
  return events;
}

double pt2_of(const PseudoJet& j) { return j.px * j.px + j.py * j.py; }

void print_jets(const std::vector<PseudoJet>& jets, bool cartesian) {
  std::cout << std::fixed << std::setprecision(8);
  int i = 0;
  for (const PseudoJet& j : jets) {
    std::cout << std::setw(5) << i++;
    if (cartesian) {
      std::cout << std::setw(16) << j.px << std::setw(16) << j.py << std::setw(16) << j.pz << std::setw(16) << j.E;
    } else {
      // rapidity and azimuth as the reference prints them (main.cc:96-111)
      const double pt = std::hypot(j.px, j.py);
      double phi = std::atan2(j.py, j.px);
      while (phi > 2 * M_PI) phi -= 2 * M_PI;
      while (phi < 0.) phi += 2 * M_PI;
      const double m2 = std::max(0.0, (j.E + j.pz) * (j.E - j.pz) - pt * pt);
      const double epz = j.E + std::abs(j.pz);
      double eta = 0.5 * std::log((pt * pt + m2) / (epz * epz));
      if (j.pz > 0) eta = -eta;
      std::cout << std::setw(16) << eta << std::setw(16) << phi << std::setw(16) << pt;
    }
    std::cout << std::endl;
  }
  std::cout << std::endl;
}

void keep_jets(std::vector<PseudoJet>& jets, double ptmin) {
  jets.erase(std::remove_if(jets.begin(), jets.end(),
                            [ptmin](const PseudoJet& j) { return !j.isJet || pt2_of(j) < ptmin * ptmin; }),
             jets.end());
}

void sort_jets(std::vector<PseudoJet>& jets) {
  std::sort(jets.begin(), jets.end(), [](const PseudoJet& a, const PseudoJet& b) { return pt2_of(a) > pt2_of(b); });
}

void print_summary(size_t n_particles, size_t n_jets, double ptmin, double sum, double sum2, long reps, bool csv) {
  std::cout << std::defaultfloat;
  if (!csv)
    std::cout << "clustered " << n_particles << " particles into " << n_jets << " jets above " << ptmin << " GeV";
  else
    std::cout << n_particles << ',' << n_jets << ',';
  std::cout << std::fixed;
  const double mean = sum / reps;
  std::streamsize old;
  if (reps > 1) {
    const double sigma = std::sqrt((sum2 - sum * sum / reps) / (reps - 1));
    old = std::cout.precision(std::max((int)-std::log10(sigma / 2.) + 1, 0));
    if (!csv)
      std::cout << " in " << mean << " +/- " << sigma << " ms" << std::endl;
    else
      std::cout << mean << ',' << sigma << std::endl;
  } else {
    old = std::cout.precision(1);
    if (!csv)
      std::cout << " in " << mean << " ms" << std::endl;
    else
      std::cout << mean << std::endl;
  }
  std::cout.precision(old);
  std::cout << std::defaultfloat;
}

void print_found(size_t n_jets, double ptmin, float ms) {
  if (ptmin > 0.)
    std::cout << "found " << n_jets << " jets above " << ptmin << " GeV in " << ms << " ms" << std::endl;
  else
    std::cout << "found " << n_jets << " jets in " << ms << " ms" << std::endl;
}

// Every event of the stream in one batched call.
int run_batch(std::istream& in, const Options& o) {
  std::vector<PseudoJet> ev;
  std::vector<std::vector<PseudoJet>> events;
  while (read_events(in, ev, o.combine == 0 ? 0 : o.combine)) events.push_back(ev);
  std::vector<int64_t> offsets(1, 0);
  std::vector<double> p4;
  for (const auto& e : events) {
    for (const PseudoJet& p : e) p4.insert(p4.end(), {p.px, p.py, p.pz, p.E});
    offsets.push_back(offsets.back() + (int64_t)e.size());
  }
  const int64_t total = offsets.back();
  const int n_events = (int)events.size();
  std::vector<double> jets(4 * std::max<int64_t>(total, 1));
  std::vector<int32_t> labels(std::max<int64_t>(total, 1)), n_jets(std::max(n_events, 1));
  fjg_ctx* ctx = nullptr;
  if (fjg_ctx_create(0, &ctx) != FJG_OK) {
    std::cerr << fjg_last_error(nullptr) << std::endl;
    return 1;
  }
  fjg_outputs out{jets.data(), labels.data(), n_jets.data(), nullptr, nullptr};
  double sum = 0., sum2 = 0.;
  const long reps = std::max(o.repetitions, 1L);
  for (long k = 0; k < reps; ++k) {
    cudaEvent_t start, stop;
    check(cudaEventCreate(&start), "cudaEventCreate");
    check(cudaEventCreate(&stop), "cudaEventCreate");
    check(cudaEventRecord(start, (cudaStream_t)fjg_ctx_stream(ctx)), "cudaEventRecord");
    const fjg_status st =
        fjg_cluster_batch_host(ctx, p4.data(), offsets.data(), n_events, nullptr, (int)o.algo, nullptr, o.r, &out);
    if (st != FJG_OK) {
      std::cerr << fjg_status_string(st) << ": " << fjg_last_error(ctx) << std::endl;
      fjg_ctx_destroy(ctx);
      return 1;
    }
    check(cudaEventRecord(stop, (cudaStream_t)fjg_ctx_stream(ctx)), "cudaEventRecord");
    check(cudaEventSynchronize(stop), "cudaEventSynchronize");
    float ms;
    check(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
    sum += ms;
    sum2 += (double)ms * ms;
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
  }
  size_t total_jets = 0;
  for (int e = 0; e < n_events; ++e) {
    std::vector<PseudoJet> js;
    for (int k = 0; k < n_jets[e]; ++k) {
      const double* q = &jets[4 * (offsets[e] + k)];
      js.push_back({labels[offsets[e] + k], true, q[0], q[1], q[2], q[3]});
    }
    keep_jets(js, o.ptmin);
    sort_jets(js);
    total_jets += js.size();
    if (!o.csv) {
      std::cout << "found " << events[e].size() << " particles" << std::endl;
      print_jets(js, o.cartesian);
    }
  }
  print_summary((size_t)total, total_jets, o.ptmin, sum, sum2, reps, o.csv);
  fjg_ctx_destroy(ctx);
  return 0;
}

}  // namespace

int main(int argc, const char* argv[]) {
  Options o;
  if (!parse(argc, argv, o)) return 1;

  check(cudaSetDevice(0), "cudaSetDevice");
  cudaDeviceProp prop;
  check(cudaGetDeviceProperties(&prop, 0), "cudaGetDeviceProperties");
  std::cout << "Running on CUDA device " << prop.name << std::endl;
  int smem = 0;
  check(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlock, 0), "cudaDeviceGetAttribute");
  std::cout << "  - maximum shared memory per block: " << smem / 1024 << " kB" << std::endl;

  std::ifstream file(o.filename);
  std::istream& in = o.filename.empty() ? std::cin : file;
  if (o.batch) return run_batch(in, o);

  std::vector<PseudoJet> particles, jets;
  long events;
  while ((events = read_events(in, particles, o.combine))) {
    if (!o.csv) {
      std::cout << "found " << particles.size() << " particles";
      if (o.combine != 1) std::cout << " in " << events << (events == 1 ? " event" : " events");
      std::cout << std::endl;
    }
    PseudoJet* d_particles = nullptr;
    check(cudaMalloc(&d_particles, sizeof(PseudoJet) * particles.size()), "cudaMalloc");
    cudaEvent_t start, stop;
    check(cudaEventCreate(&start), "cudaEventCreate");
    check(cudaEventCreate(&stop), "cudaEventCreate");
    double sum = 0., sum2 = 0.;
    for (long step = 0; o.repetitions == 0 || step < o.repetitions; ++step) {
      check(cudaEventRecord(start), "cudaEventRecord");
      check(cudaMemcpy(d_particles, particles.data(), sizeof(PseudoJet) * particles.size(), cudaMemcpyDefault),
            "cudaMemcpy");
      cluster(d_particles, (int)particles.size(), o.algo, o.r);
      jets.resize(particles.size());
      check(cudaMemcpy(jets.data(), d_particles, sizeof(PseudoJet) * jets.size(), cudaMemcpyDefault), "cudaMemcpy");
      check(cudaEventRecord(stop), "cudaEventRecord");
      check(cudaEventSynchronize(stop), "cudaEventSynchronize");
      float ms;
      check(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
      sum += ms;
      sum2 += (double)ms * ms;
      keep_jets(jets, o.ptmin);
      if (!o.csv) {
        print_found(jets.size(), o.ptmin, ms);
        sort_jets(jets);
      }
    }
    check(cudaFree(d_particles), "cudaFree");
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    if (!o.csv) print_jets(jets, o.cartesian);
    print_summary(particles.size(), jets.size(), o.ptmin, sum, sum2, o.repetitions, o.csv);
  }
  return 0;
}

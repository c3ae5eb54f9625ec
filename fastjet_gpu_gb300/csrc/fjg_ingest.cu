// Reader of the reference driver's event text into CSR arrays
// (fjg_parse_events in fastjet_gb300.h).  Host code only.
//
// The format is the one main.cc:34-70 reads: one particle per line,
// "px py pz E" (whitespace separated, anything after the fourth number
// ignored); an event is a maximal run of such lines; a line that is empty or
// starts with '#' ends an event (and runs of them are skipped); any other line
// is an error (main.cc:55-58 throws); a final line without a newline is not
// read (the reference's getline loop stops at end of file before parsing it).
// Numbers are read as istream >> double
// reads them (correctly rounded decimal, optional sign, no inf/nan): here with
// std::from_chars, also correctly rounded, so the values are the same bits.
//
// The text is cut into chunks at line ends, one per thread; each thread
// classifies and parses its lines, recording where events start inside the
// chunk.  Whether a chunk's first particle continues the previous chunk's
// event is settled from the neighbouring chunks afterwards, and the threads
// then copy their rows into the output at their prefix offsets.
#include <charconv>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "fjg_context.h"

using fjg::set_error;

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// One number as istream >> double reads it; returns the end or nullptr.
inline const char* read_number(const char* p, const char* end, double* out) {
  while (p < end && is_space(*p)) ++p;
  if (p >= end) return nullptr;
  const char* q = p;
  bool neg = false;
  if (*q == '+' || *q == '-') {
    neg = *q == '-';
    ++q;
  }
  if (q >= end || !((*q >= '0' && *q <= '9') || *q == '.')) return nullptr;  // no inf / nan
  double v = 0.0;
  const auto r = std::from_chars(q, end, v, std::chars_format::general);
  if (r.ec != std::errc()) return nullptr;
  *out = neg ? -v : v;
  return r.ptr;
}

enum LineKind { kParticle, kSeparator, kBad };

inline LineKind classify(const char* b, const char* e, double* v) {
  if (b == e || *b == '#') return kSeparator;
  const char* p = b;
  for (int k = 0; k < 4; ++k) {
    p = read_number(p, e, v + k);
    if (!p) return kBad;
  }
  return kParticle;
}

struct Chunk {
  const char* b = nullptr;
  const char* e = nullptr;
  std::vector<double> rows;      // 4 per particle line
  std::vector<int64_t> starts;   // local rows that begin an event inside the chunk
  bool has_lines = false;
  bool first_is_particle = false;
  bool last_is_particle = false;
  int64_t newlines = 0;          // '\n' in [b, e)
  int64_t bad_line = -1;         // first rejected line, 0-based within the chunk
};

void parse_chunk(Chunk& c) {
  const char* p = c.b;
  int64_t line = 0;
  bool prev_particle = false;
  double v[4];
  while (p < c.e) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(c.e - p)));
    if (!nl) break;  // a final line without a newline is not read (main.cc:47: getline(...).good())
    const char* le = nl;
    const LineKind k = classify(p, le, v);
    if (k == kBad) {
      if (c.bad_line < 0) c.bad_line = line;
    } else if (k == kParticle) {
      if (line > 0 && !prev_particle) c.starts.push_back(static_cast<int64_t>(c.rows.size() / 4));
      c.rows.insert(c.rows.end(), v, v + 4);
    }
    if (line == 0) c.first_is_particle = k == kParticle;
    c.last_is_particle = k == kParticle;
    prev_particle = k == kParticle;
    c.has_lines = true;
    ++line;
    ++c.newlines;
    p = nl + 1;
  }
}

}  // namespace

extern "C" {

fjg_status fjg_parse_events(const char* text, size_t len, int threads, double* particles, int64_t max_particles,
                            int64_t* offsets, int64_t max_offsets, int64_t* n_particles, int64_t* n_events,
                            int64_t* error_line) {
  if (!n_particles || !n_events || (len > 0 && !text) || max_particles < 0 || max_offsets < 0)
    return set_error(nullptr, FJG_EINVAL, "fjg_parse_events: bad arguments");
  if (error_line) *error_line = 0;
  // chunks of at least 1 MiB, cut after a '\n'
  int T = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  if (T < 1) T = 1;
  const size_t min_chunk = size_t(1) << 20;
  if (static_cast<size_t>(T) > len / min_chunk + 1) T = static_cast<int>(len / min_chunk + 1);
  std::vector<Chunk> chunks(static_cast<size_t>(T));
  const char* end = text + len;
  const char* cur = text;
  for (int k = 0; k < T; ++k) {
    chunks[k].b = cur;
    const char* target = (k == T - 1) ? end : text + len / T * (k + 1);
    if (target < cur) target = cur;
    const char* nl = target < end ? static_cast<const char*>(std::memchr(target, '\n', static_cast<size_t>(end - target)))
                                  : nullptr;
    cur = (k == T - 1 || !nl) ? end : nl + 1;
    chunks[k].e = cur;
  }
  if (T == 1) {
    parse_chunk(chunks[0]);
  } else {
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(T));
    for (int k = 0; k < T; ++k) pool.emplace_back(parse_chunk, std::ref(chunks[k]));
    for (auto& t : pool) t.join();
  }
  // the first rejected line, counted from 1 over the whole text
  int64_t lines_before = 0;
  for (const Chunk& c : chunks) {
    if (c.bad_line >= 0) {
      if (error_line) *error_line = lines_before + c.bad_line + 1;
      return set_error(nullptr, FJG_EINVAL,
                       "fjg_parse_events: line " + std::to_string(lines_before + c.bad_line + 1) +
                           " is neither a particle (px py pz E), empty, nor a comment");
    }
    lines_before += c.newlines;
  }
  // event starts across chunk boundaries, then prefix sums
  int64_t rows = 0, events = 0;
  bool prev_particle = false;
  std::vector<int64_t> row0(chunks.size()), ev0(chunks.size());
  std::vector<char> first_starts(chunks.size(), 0);
  for (size_t k = 0; k < chunks.size(); ++k) {
    Chunk& c = chunks[k];
    row0[k] = rows;
    ev0[k] = events;
    if (!c.has_lines) continue;
    first_starts[k] = c.first_is_particle && !prev_particle;
    rows += static_cast<int64_t>(c.rows.size() / 4);
    events += static_cast<int64_t>(c.starts.size()) + first_starts[k];
    prev_particle = c.last_is_particle;
  }
  *n_particles = rows;
  *n_events = events;
  if (rows > max_particles || events + 1 > max_offsets || !offsets || (rows > 0 && !particles))
    return set_error(nullptr, FJG_ETOOBIG,
                     "fjg_parse_events: output capacity too small (" + std::to_string(rows) + " particles, " +
                         std::to_string(events + 1) + " offsets needed)");
  auto fill = [&](size_t k) {
    const Chunk& c = chunks[k];
    if (!c.rows.empty()) std::memcpy(particles + 4 * row0[k], c.rows.data(), c.rows.size() * sizeof(double));
    int64_t e = ev0[k];
    if (first_starts[k]) offsets[e++] = row0[k];
    for (int64_t s : c.starts) offsets[e++] = row0[k] + s;
  };
  if (chunks.size() == 1) {
    fill(0);
  } else {
    std::vector<std::thread> pool;
    for (size_t k = 0; k < chunks.size(); ++k) pool.emplace_back(fill, k);
    for (auto& t : pool) t.join();
  }
  offsets[events] = rows;
  return FJG_OK;
}

}  // extern "C"

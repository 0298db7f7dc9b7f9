// Fast reader of MPS files: the Model that samaya::read_mps (reference src/io/mps_reader.cpp)
// builds, for linear models, read by several host threads. Like samaya's reader it reads free MPS
// first and, where that fails, fixed MPS (data fields in fixed columns, names with spaces).
//
// The text is cut at its section headers (lines that start with neither a blank nor '*'; found by
// one parallel scan). Each section's data lines are cut into line-aligned byte ranges, one thread
// per range. ROWS and COLUMNS names go into open-addressing tables of views into the text, filled
// by compare-and-swap so that the first occurrence in file order owns a name. Lines that change
// state line by line (bounds, right-hand sides, ranges) are parsed in parallel into records and
// applied in file order. The columns' entries are kept per run of consecutive lines of one column
// and become the CSC arrays in two parallel passes (sort each column by row, add duplicates and
// drop exact zeros; then copy to the prefix-summed offsets).
//
// What the reference's free-MPS parse does, and this reader therefore does, line by line:
// numbers through std::from_chars after one leading '+' is stripped, |v| >= 1e30 infinite
// (mps_reader.cpp:112-123); the first N row is the objective unless OBJNAME names one, other N
// rows are dropped (:225-244); an RHS entry on the objective sets the offset to minus its value
// (:318-344); columns default to [0, +inf), UP < 0 on a column without a set lower bound makes the
// lower -inf (:346-400); ranges as in :452-476; the matrix summed as SparseMatrix::from_triplets
// sums it (reference src/linalg/sparse_matrix.cpp:15-46); the checks of Model::validate
// (reference src/core/model.cpp:59-104). One order is left open: three or more entries for the
// same (row, column) are added in file order here, where from_triplets adds them in the order its
// unstable sort leaves them (two entries give the same sum either way).
//
// The quadratic sections (QUADOBJ, QMATRIX, QSECTION, QCMATRIX) are declined (kUnsupported), and
// input that neither free nor fixed MPS reads is a kParseError with the free reading's message
// and line: in both cases the caller hands the file to samaya's own reader.
#include "sg_mps.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>
#include <new>
#include <string>
#include <string_view>
#include <system_error>
#include <thread>
#include <utility>
#include <vector>

namespace sg {
namespace {

using std::string_view;

constexpr double kInfiniteBound = 1e30;  // samaya's kInfiniteBound (include/samaya/types.hpp:16)
constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int kMaxThreads = 64;
constexpr size_t kBytesPerThread = size_t{1} << 20;  // automatic threads: one per MiB of a section
constexpr int64_t kMaxIndex = std::numeric_limits<int32_t>::max();

struct Failure {
  MpsStatus status;
  const char* at;  // the failing line, or nullptr
  std::string message;
};

[[noreturn]] void fail(const char* at, std::string message,
                       MpsStatus status = MpsStatus::kParseError) {
  throw Failure{status, at, std::move(message)};
}

// Runs f(0..threads-1) on that many threads (the caller's thread included); a thread that cannot
// be started runs on the caller's thread. The first exception, in thread order, is rethrown here
// after every thread has ended.
template <class F>
void run_threads(int threads, const F& f) {
  std::vector<std::exception_ptr> errors(static_cast<size_t>(std::max(threads, 1)));
  auto body = [&](int t) {
    try {
      f(t);
    } catch (...) {
      errors[t] = std::current_exception();
    }
  };
  if (threads <= 1) {
    body(0);
  } else {
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(threads - 1));
    int started = 1;
    try {
      for (; started < threads; ++started) pool.emplace_back(body, started);
    } catch (const std::system_error&) {
    }
    for (int t = started; t < threads; ++t) body(t);
    body(0);
    for (auto& th : pool) th.join();
  }
  for (const std::exception_ptr& e : errors) {
    if (e) std::rethrow_exception(e);
  }
}

inline bool blank(char c) { return c == ' ' || c == '\t'; }

struct Tokens {
  static constexpr int kKept = 8;
  string_view t[kKept];
  int n = 0;  // all tokens of the line; the first kKept are kept
};

inline void tokenize(const char* p, const char* e, Tokens& tk) {
  tk.n = 0;
  while (p < e) {
    while (p < e && blank(*p)) ++p;
    const char* s = p;
    while (p < e && !blank(*p)) ++p;
    if (p > s) {
      if (tk.n < Tokens::kKept) tk.t[tk.n] = string_view(s, static_cast<size_t>(p - s));
      ++tk.n;
    }
  }
}

// Fixed MPS (mps_reader.cpp:100-115): the data fields sit in columns 2-3, 5-12, 15-22, 25-36,
// 40-47 and 50-61; each is trimmed of blanks and an empty one is skipped, which leaves the token
// layout of free MPS. Names may then contain spaces.
inline void tokenize_fixed(const char* p, const char* e, Tokens& tk) {
  static constexpr size_t kStart[] = {1, 4, 14, 24, 39, 49};
  static constexpr size_t kEnd[] = {3, 12, 22, 36, 47, 61};
  const size_t len = static_cast<size_t>(e - p);
  tk.n = 0;
  for (size_t f = 0; f < 6 && kStart[f] < len; ++f) {
    const char* a = p + kStart[f];
    const char* b = p + std::min(kEnd[f], len);
    while (a < b && blank(*a)) ++a;
    while (b > a && blank(b[-1])) --b;
    if (b > a) {
      if (tk.n < Tokens::kKept) tk.t[tk.n] = string_view(a, static_cast<size_t>(b - a));
      ++tk.n;
    }
  }
}

// Calls f(begin, end) for each line of [b, e) (b at a line start, e at a line start or the end of
// the text) without its '\n' and one trailing '\r'; stops when f returns false.
template <class F>
void for_lines(const char* b, const char* e, F&& f) {
  while (b < e) {
    const char* nl = static_cast<const char*>(std::memchr(b, '\n', static_cast<size_t>(e - b)));
    const char* le = nl ? nl : e;
    const char* x = le;
    if (x > b && x[-1] == '\r') --x;
    if (!f(b, x)) return;
    b = nl ? nl + 1 : e;
  }
}

bool iequals(string_view a, string_view b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i) {
    const char x = (a[i] >= 'A' && a[i] <= 'Z') ? static_cast<char>(a[i] + 32) : a[i];
    const char y = (b[i] >= 'A' && b[i] <= 'Z') ? static_cast<char>(b[i] + 32) : b[i];
    if (x != y) return false;
  }
  return true;
}

// Exact powers of ten as doubles (10^0 .. 10^22 are all exactly representable).
constexpr double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                               1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// Short decimals ([-]digits[.digits][(e|E)[+-]digits]) by Clinger's fast path (W. D. Clinger,
// "How to Read Floating Point Numbers Accurately", PLDI 1990): with the digits as an integer
// M < 2^53 and a power of ten 10^k, |k| <= 22, both M and 10^|k| are exact doubles, so one IEEE
// multiplication or division gives the correctly rounded value, the one std::from_chars returns.
// Returns false for every other token, which then goes to std::from_chars.
inline bool parse_short_decimal(const char* p, const char* e, double* v) {
  bool neg = false;
  if (p < e && *p == '-') {
    neg = true;
    ++p;
  }
  uint64_t mant = 0;
  int digits = 0, frac = 0;
  const char* q = p;
  while (q < e && static_cast<unsigned>(*q - '0') < 10) {
    mant = mant * 10 + static_cast<unsigned>(*q - '0');
    ++digits;
    ++q;
  }
  if (q < e && *q == '.') {
    ++q;
    while (q < e && static_cast<unsigned>(*q - '0') < 10) {
      mant = mant * 10 + static_cast<unsigned>(*q - '0');
      ++digits;
      ++frac;
      ++q;
    }
  }
  if (digits == 0 || digits > 19) return false;
  int exp10 = 0;
  if (q < e && (*q == 'e' || *q == 'E')) {
    ++q;
    bool eneg = false;
    if (q < e && (*q == '+' || *q == '-')) eneg = *q++ == '-';
    int ed = 0;
    while (q < e && static_cast<unsigned>(*q - '0') < 10 && ed < 4) {
      exp10 = exp10 * 10 + (*q - '0');
      ++ed;
      ++q;
    }
    if (ed == 0) return false;
    if (eneg) exp10 = -exp10;
  }
  if (q != e) return false;
  const int k = exp10 - frac;
  if (mant > (uint64_t{1} << 53) || k < -22 || k > 22) return false;
  double x = static_cast<double>(mant);
  x = k >= 0 ? x * kPow10[k] : x / kPow10[-k];
  *v = neg ? -x : x;
  return true;
}

inline bool parse_number(string_view s, double* v) {
  if (!s.empty() && s.front() == '+') s.remove_prefix(1);
  double x = 0.0;
  // A token of 18 or more characters rarely fits the fast path's 2^53 mantissa (17-digit
  // values are written that long): it goes straight to from_chars, scanned once.
  if (s.size() >= 18 || !parse_short_decimal(s.data(), s.data() + s.size(), &x)) {
    const auto r = std::from_chars(s.data(), s.data() + s.size(), x);
    if (r.ec != std::errc() || r.ptr != s.data() + s.size()) return false;
  }
  if (x >= kInfiniteBound) {
    x = kInf;
  } else if (x <= -kInfiniteBound) {
    x = -kInf;
  }
  *v = x;
  return true;
}

// Hash of a name, eight bytes at a time (an internal table key only).
inline uint32_t hash_name(const char* p, size_t n) {
  uint64_t h = 0x9E3779B97F4A7C15ull ^ (n * 0xD6E8FEB86659FD93ull);
  while (n >= 8) {
    uint64_t w;
    std::memcpy(&w, p, 8);
    h = (h ^ w) * 0xFF51AFD7ED558CCDull;
    h ^= h >> 32;
    p += 8;
    n -= 8;
  }
  uint64_t w = 0;
  std::memcpy(&w, p, n);
  h = (h ^ w) * 0xC4CEB9FE1A85EC53ull;
  h ^= h >> 29;
  h *= 0x9E3779B97F4A7C15ull;
  return static_cast<uint32_t>(h ^ (h >> 32));
}

struct Key {
  const char* p;
  uint32_t len;
  uint32_t hash;
  string_view view() const { return string_view(p, len); }
};

inline Key make_key(string_view s) {
  if (s.size() > std::numeric_limits<uint32_t>::max()) fail(s.data(), "name too long");
  return Key{s.data(), static_cast<uint32_t>(s.size()), hash_name(s.data(), s.size())};
}

inline bool same(const Key& a, const Key& b) {
  return a.hash == b.hash && a.len == b.len && std::memcmp(a.p, b.p, a.len) == 0;
}

// Open-addressing table of key ids (linear probing, at most half full). insert_range inserts
// ids in parallel; of two ids with the same name the smaller keeps the slot and the other is
// flagged in `lost`.
class NameTable {
 public:
  void insert_range(const Buffer<Key>& keys, size_t b, size_t e, uint8_t* lost, int threads) {
    if (2 * e > cap_) {
      size_t cap = 1024;
      while (cap < 2 * e) cap *= 2;
      slot_.reset(new std::atomic<int32_t>[cap]);
      cap_ = cap;
      mask_ = cap - 1;
      fill(threads);
      b = 0;  // every earlier id goes into the new table (the same ids win)
    }
    const size_t count = e - b;
    const int parts = static_cast<int>(std::max<size_t>(1, std::min<size_t>(threads, count / 4096)));
    run_threads(parts, [&](int t) {
      const size_t lo = b + count * t / parts, hi = b + count * (t + 1) / parts;
      for (size_t id = lo; id < hi; ++id) insert(keys.data(), static_cast<int32_t>(id), lost);
    });
  }

  // The id that owns the name, or -1.
  int32_t find(const Key* keys, const Key& k) const {
    if (cap_ == 0) return -1;
    size_t i = k.hash & mask_;
    for (;;) {
      const int32_t cur = slot_[i].load(std::memory_order_relaxed);
      if (cur < 0) return -1;
      if (same(keys[cur], k)) return cur;
      i = (i + 1) & mask_;
    }
  }

 private:
  void fill(int threads) {
    const int parts = static_cast<int>(std::max<size_t>(1, std::min<size_t>(threads, cap_ >> 16)));
    run_threads(parts, [&](int t) {
      for (size_t i = cap_ * t / parts, e = cap_ * (t + 1) / parts; i < e; ++i) {
        slot_[i].store(-1, std::memory_order_relaxed);
      }
    });
  }

  void insert(const Key* keys, int32_t id, uint8_t* lost) {
    const Key& k = keys[id];
    size_t i = k.hash & mask_;
    for (;;) {
      int32_t cur = slot_[i].load(std::memory_order_acquire);
      if (cur < 0) {
        if (slot_[i].compare_exchange_weak(cur, id, std::memory_order_acq_rel)) return;
        continue;
      }
      if (same(keys[cur], k)) {
        if (id < cur) {
          if (slot_[i].compare_exchange_weak(cur, id, std::memory_order_acq_rel)) {
            lost[cur] = 1;
            return;
          }
          continue;
        }
        lost[id] = 1;
        return;
      }
      i = (i + 1) & mask_;
    }
  }

  std::unique_ptr<std::atomic<int32_t>[]> slot_;
  size_t cap_ = 0;
  size_t mask_ = 0;
};

// First error of a parallel pass, in file order.
struct ChunkError {
  const char* at = nullptr;
  std::string message;
  bool fail(const char* p, std::string m) {
    at = p;
    message = std::move(m);
    return false;
  }
};

template <class Chunk>
void rethrow_first(const std::vector<Chunk>& chunks) {
  for (const Chunk& c : chunks) {
    if (c.error.at != nullptr) fail(c.error.at, c.error.message);
  }
}

// A run of consecutive COLUMNS lines of one column within a chunk.
struct Run {
  uint32_t e0, ne;  // entries [e0, e0 + ne) of the chunk's rows / vals
  uint32_t o0, no;  // objective values [o0, o0 + no) of the chunk's objv
  int8_t state;     // integer marker state at the run's first line: -1 = the chunk's start state
};

struct ColChunk {
  std::vector<Key> keys;  // one per run
  std::vector<Run> runs;
  std::vector<int32_t> rows;
  std::vector<double> vals;
  std::vector<double> objv;
  int8_t end_state = -1;
  bool clean = true;  // every run's rows strictly increase and no value is zero
  ChunkError error;
};

struct Place {
  uint32_t chunk, run;
};

enum class Section { kNone, kObjSense, kObjName, kRows, kColumns, kRhs, kRanges, kBounds, kEnd };

enum BoundType : uint8_t { kUP, kUI, kLO, kLI, kFX, kFR, kMI, kPL, kBV };

constexpr int32_t kObjectiveRow = -1;
constexpr int32_t kFreeRow = -2;
constexpr int32_t kUnknownRow = -3;

// With SG_MPS_PHASES set (to anything but "0"), the reader prints the wall time of each phase to
// stderr: a diagnostic for profiling the reader.
class PhaseClock {
 public:
  PhaseClock() {
    const char* e = std::getenv("SG_MPS_PHASES");
    on_ = e != nullptr && *e != '\0' && std::strcmp(e, "0") != 0;
    last_ = std::chrono::steady_clock::now();
  }
  void mark(const char* phase) {
    if (!on_) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "sg_mps %-10s %9.2f ms\n", phase,
                 std::chrono::duration<double, std::milli>(now - last_).count());
    last_ = now;
  }

 private:
  bool on_ = false;
  std::chrono::steady_clock::time_point last_;
};

class Reader {
 public:
  Reader(const char* text, size_t len, int threads, bool fixed)
      : text_(text), len_(len), fixed_(fixed) {
    const unsigned hw = std::thread::hardware_concurrency();
    hw_threads_ = std::max(1, std::min(kMaxThreads, static_cast<int>(hw == 0 ? 1 : hw)));
    forced_ = threads > 0 ? std::min(threads, kMaxThreads) : 0;
  }

  void read(MpsModel* out) {
    const char* end = text_ + len_;
    const std::vector<const char*> headers = find_headers();
    clock_.mark("headers");
    no_data(text_, headers.empty() ? end : headers[0]);
    for (size_t k = 0; k < headers.size(); ++k) {
      const char* h = headers[k];
      const char* nl = static_cast<const char*>(std::memchr(h, '\n', static_cast<size_t>(end - h)));
      const char* hl = nl ? nl : end;
      if (hl > h && hl[-1] == '\r') --hl;
      const char* body = nl ? nl + 1 : end;
      const char* body_end = k + 1 < headers.size() ? headers[k + 1] : end;
      Tokens tk;
      tokenize(h, hl, tk);
      const Section s = header(tk, h);
      if (s == Section::kEnd) {
        last_line_ = h;
        break;
      }
      switch (s) {
        case Section::kNone: no_data(body, body_end); break;
        case Section::kObjSense:
          each_data_line(body, body_end, [&](const Tokens& t, const char* p) { set_sense(t.t[0], p); });
          break;
        case Section::kObjName:
          each_data_line(body, body_end,
                         [&](const Tokens& t, const char* p) { set_objective_name(t.t[0], p); });
          break;
        case Section::kRows: rows(body, body_end); clock_.mark("rows"); break;
        case Section::kColumns: columns(body, body_end); break;
        case Section::kRhs: rhs(body, body_end, false); clock_.mark("rhs"); break;
        case Section::kRanges: rhs(body, body_end, true); clock_.mark("ranges"); break;
        case Section::kBounds: bounds(body, body_end); clock_.mark("bounds"); break;
        case Section::kEnd: break;
      }
    }
    finish(out);
  }

 private:
  int parts_for(size_t bytes) const {
    if (forced_ > 0) return forced_;
    return static_cast<int>(std::max<size_t>(1, std::min<size_t>(hw_threads_, bytes / kBytesPerThread)));
  }

  // Line-aligned cut of [b, e) into `parts` ranges.
  static std::vector<const char*> split_lines(const char* b, const char* e, int parts) {
    std::vector<const char*> cut(static_cast<size_t>(parts) + 1);
    cut[0] = b;
    cut[parts] = e;
    const size_t bytes = static_cast<size_t>(e - b);
    for (int t = 1; t < parts; ++t) {
      const char* p = b + bytes / parts * t + bytes % parts * t / parts;
      if (p < cut[t - 1]) p = cut[t - 1];
      if (p > b && p < e && p[-1] != '\n') {
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(e - p)));
        p = nl ? nl + 1 : e;
      }
      cut[t] = p;
    }
    return cut;
  }

  // The tokens of a data line, free or fixed.
  void tokens(const char* p, const char* q, Tokens& tk) const {
    if (fixed_) {
      tokenize_fixed(p, q, tk);
    } else {
      tokenize(p, q, tk);
    }
  }

  // The column named by a COLUMNS line, or an empty view for a line that names none (empty,
  // comment, blanks only, a marker line).
  string_view column_of(const char* p, const char* q) const {
    if (q > p && q[-1] == '\r') --q;
    if (p == q || *p == '*') return {};
    Tokens tk;
    tokens(p, q, tk);
    if (tk.n == 0 || (tk.n >= 3 && tk.t[1] == "'MARKER'")) return {};
    return tk.t[0];
  }

  // split_lines for a COLUMNS body, each cut moved on past the lines of the column it would split
  // (markers, comments and blank lines in between included), so that every run of consecutive
  // lines of one column lies in one range.
  std::vector<const char*> split_columns(const char* b, const char* e, int parts) const {
    std::vector<const char*> cut = split_lines(b, e, parts);
    for (int t = 1; t < parts; ++t) {
      const char* p = std::max(cut[t], cut[t - 1]);
      // The column of the last line before p that names one.
      string_view prev;
      for (const char* le = p; le > b && prev.empty();) {
        const char* ls = le - 1;  // ls: the '\n' ending the previous line
        while (ls > b && ls[-1] != '\n') --ls;
        prev = column_of(ls, le - 1);
        le = ls;
      }
      while (!prev.empty() && p < e) {
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(e - p)));
        const char* le = nl ? nl : e;
        const string_view name = column_of(p, le);
        if (!name.empty() && name != prev) break;
        p = nl ? nl + 1 : e;
      }
      cut[t] = p;
    }
    return cut;
  }

  // Starts of the header lines: non-empty (after one trailing '\r' is dropped), first character
  // neither a blank nor '*' (mps_reader.cpp:125-134).
  std::vector<const char*> find_headers() const {
    const char* end = text_ + len_;
    const int parts = parts_for(len_);
    std::vector<std::vector<const char*>> found(static_cast<size_t>(parts));
    run_threads(parts, [&](int t) {
      const char* b = text_ + len_ * t / parts;
      const char* e = text_ + len_ * (t + 1) / parts;
      const char* p = b;
      if (p > text_ && p[-1] != '\n') {
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(end - p)));
        p = nl ? nl + 1 : end;
      }
      while (p < e) {  // p: a line start owned by this range
        const char c = *p;
        const bool empty = c == '\n' || (c == '\r' && (p + 1 == end || p[1] == '\n'));
        if (!empty && !blank(c) && c != '*') found[t].push_back(p);
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(end - p)));
        if (!nl) break;
        p = nl + 1;
      }
    });
    std::vector<const char*> all;
    for (auto& f : found) all.insert(all.end(), f.begin(), f.end());
    return all;
  }

  template <class F>
  void each_data_line(const char* b, const char* e, F&& f) {
    Tokens tk;
    for_lines(b, e, [&](const char* p, const char* q) {
      if (p == q || *p == '*') return true;
      tokens(p, q, tk);
      if (tk.n > 0) f(tk, p);
      return true;
    });
  }

  void no_data(const char* b, const char* e) {
    each_data_line(b, e, [](const Tokens&, const char* p) { fail(p, "data line outside of a section"); });
  }

  Section header(const Tokens& tk, const char* at) {
    const string_view key = tk.t[0];
    if (key == "NAME") {
      if (tk.n > 1) name_ = std::string(tk.t[1]);
      return Section::kNone;
    }
    if (key == "OBJSENSE") {
      if (tk.n > 1) set_sense(tk.t[1], at);
      return Section::kObjSense;
    }
    if (key == "OBJNAME") {
      if (tk.n > 1) set_objective_name(tk.t[1], at);
      return Section::kObjName;
    }
    if (key == "ROWS") return Section::kRows;
    if (key == "COLUMNS") return Section::kColumns;
    if (key == "RHS") return Section::kRhs;
    if (key == "RANGES") return Section::kRanges;
    if (key == "BOUNDS") return Section::kBounds;
    if (key == "ENDATA") return Section::kEnd;
    if (key == "QUADOBJ" || key == "QMATRIX" || key == "QSECTION" || key == "QCMATRIX") {
      fail(at, "section " + std::string(key) + " (quadratic terms) is read by samaya's own reader",
           MpsStatus::kUnsupported);
    }
    if (key == "SOS" || key == "INDICATORS" || key == "CSECTION") {
      fail(at, "section " + std::string(key) + " is not supported");
    }
    fail(at, "unknown section '" + std::string(key) + "'");
  }

  void set_sense(string_view s, const char* at) {
    if (iequals(s, "MAX") || iequals(s, "MAXIMIZE")) {
      maximize_ = true;
    } else if (iequals(s, "MIN") || iequals(s, "MINIMIZE")) {
      maximize_ = false;
    } else {
      fail(at, "unknown objective sense '" + std::string(s) + "'");
    }
  }

  void set_objective_name(string_view s, const char* at) {
    if (!row_keys_.empty()) fail(at, "OBJNAME must precede ROWS");
    objective_ = std::string(s);
  }

  // kObjectiveRow, kFreeRow, a row index, or kUnknownRow.
  int32_t find_row(string_view name) const {
    if (name.size() == objective_.size() && name == objective_) return kObjectiveRow;
    const int32_t id = row_table_.find(row_keys_.data(), make_key(name));
    return id < 0 ? kUnknownRow : row_val_[id];
  }

  // The column index, or -1.
  int32_t find_col(string_view name) const {
    const int32_t id = col_table_.find(col_keys_.data(), make_key(name));
    return id < 0 ? -1 : cand_col_[id];
  }

  static bool named(const Key& k, string_view name) {
    return k.len == name.size() && std::memcmp(k.p, name.data(), k.len) == 0;
  }

  // find_col, trying the column after `*last` (and `*last` itself) first: bound lines mostly
  // follow the column order, and comparing that column's name reads the text in order.
  int32_t find_col_after(string_view name, int32_t* last) const {
    for (int32_t c : {*last + 1, *last}) {
      if (c >= 0 && c < n_ && named(col_keys_[col_cand_[c]], name)) return *last = c;
    }
    const int32_t c = find_col(name);
    if (c >= 0) *last = c;
    return c;
  }

  // find_row with the same guess for right-hand sides and ranges listed in row order.
  int32_t find_row_after(string_view name, int32_t* last) const {
    if (name.size() == objective_.size() && name == objective_) return kObjectiveRow;
    for (int32_t r : {*last + 1, *last}) {
      if (r >= 0 && r < m_ && named(row_keys_[row_name_id_[r]], name)) return *last = r;
    }
    const int32_t r = find_row(name);
    if (r >= 0) *last = r;
    return r;
  }

  // ---- ROWS (mps_reader.cpp:225-244) ----
  void rows(const char* b, const char* e) {
    struct Chunk {
      std::vector<Key> keys;
      std::vector<char> kinds;
      ChunkError error;
    };
    const int parts = parts_for(static_cast<size_t>(e - b));
    const std::vector<const char*> cut = split_lines(b, e, parts);
    std::vector<Chunk> ch(static_cast<size_t>(parts));
    run_threads(parts, [&](int t) {
      Chunk& c = ch[t];
      Tokens tk;
      for_lines(cut[t], cut[t + 1], [&](const char* p, const char* q) {
        if (p == q || *p == '*') return true;
        tokens(p, q, tk);
        if (tk.n == 0) return true;
        if (tk.n < 2) return c.error.fail(p, "ROWS entry needs a type and a name");
        const string_view type = tk.t[0];
        char kind;
        if (iequals(type, "N")) {
          kind = 'N';
        } else if (iequals(type, "E")) {
          kind = 'E';
        } else if (iequals(type, "L")) {
          kind = 'L';
        } else if (iequals(type, "G")) {
          kind = 'G';
        } else {
          return c.error.fail(p, "unknown row type '" + std::string(type) + "'");
        }
        c.keys.push_back(make_key(tk.t[1]));
        c.kinds.push_back(kind);
        return true;
      });
    });
    // A malformed line fails the read, but a duplicate name on an earlier line fails it first
    // (samaya stops at the first of the two): the records of the ranges up to the failing one,
    // which all precede the failing line, still go through the duplicate check below.
    size_t failed = ch.size();
    for (size_t t = 0; t < ch.size() && failed == ch.size(); ++t) {
      if (ch[t].error.at != nullptr) failed = t;
    }
    const size_t base = row_keys_.size();
    for (size_t t = 0; t < ch.size() && t <= failed; ++t) {
      const Chunk& c = ch[t];
      for (size_t i = 0; i < c.keys.size(); ++i) {
        const Key& k = c.keys[i];
        int32_t v;
        if (c.kinds[i] == 'N') {
          if (objective_.empty()) objective_ = std::string(k.view());
          v = k.view() == objective_ ? kObjectiveRow : kFreeRow;
        } else {
          if (m_ >= kMaxIndex) fail(k.p, "more than 2^31 - 1 rows", MpsStatus::kTooLarge);
          v = m_++;
          row_kind_.push_back(c.kinds[i]);
          row_name_id_.push_back(static_cast<int32_t>(row_keys_.size()));
        }
        row_keys_.push_back(k);
        row_val_.push_back(v);
      }
    }
    if (row_keys_.size() > static_cast<size_t>(kMaxIndex)) {
      fail(nullptr, "too many rows", MpsStatus::kTooLarge);
    }
    row_lost_.resize(row_keys_.size());
    std::fill(row_lost_.begin() + static_cast<std::ptrdiff_t>(base), row_lost_.end(), uint8_t{0});
    row_table_.insert_range(row_keys_, base, row_keys_.size(), row_lost_.data(), threads_for(row_keys_.size() - base));
    for (size_t id = base; id < row_keys_.size(); ++id) {
      if (row_lost_[id]) {
        fail(row_keys_[id].p, "duplicate row '" + std::string(row_keys_[id].view()) + "'");
      }
    }
    if (failed < ch.size()) fail(ch[failed].error.at, ch[failed].error.message);
  }

  int threads_for(size_t items) const {
    if (forced_ > 0) return forced_;
    return static_cast<int>(std::max<size_t>(1, std::min<size_t>(hw_threads_, items / 16384)));
  }

  // ---- COLUMNS (mps_reader.cpp:281-302) ----
  void parse_columns(const char* b, const char* e, ColChunk& c) const {
    Tokens tk;
    int8_t state = -1;
    const size_t bytes = static_cast<size_t>(e - b);
    c.rows.reserve(bytes / 20);
    c.vals.reserve(bytes / 20);
    c.keys.reserve(bytes / 40);
    c.runs.reserve(bytes / 40);
    c.objv.reserve(bytes / 40);
    for_lines(b, e, [&](const char* p, const char* q) {
      if (p == q || *p == '*') return true;
      tokens(p, q, tk);
      if (tk.n == 0) return true;
      if (tk.n >= 3 && tk.t[1] == "'MARKER'") {
        if (tk.t[2] == "'INTORG'") {
          state = 1;
        } else if (tk.t[2] == "'INTEND'") {
          state = 0;
        } else {
          return c.error.fail(p, "unknown marker " + std::string(tk.t[2]));
        }
        return true;
      }
      if (tk.n != 3 && tk.n != 5) return c.error.fail(p, "COLUMNS entry needs 3 or 5 fields");
      // A line that goes on with the last run's column is told by its bytes, without a hash.
      const string_view name = tk.t[0];
      if (c.runs.empty() || c.keys.back().len != name.size() ||
          std::memcmp(c.keys.back().p, name.data(), name.size()) != 0) {
        if (c.rows.size() > std::numeric_limits<uint32_t>::max() - 2 ||
            c.objv.size() > std::numeric_limits<uint32_t>::max() - 2) {
          return c.error.fail(p, "too many entries in one range");
        }
        c.keys.push_back(make_key(name));
        c.runs.push_back(Run{static_cast<uint32_t>(c.rows.size()), 0,
                             static_cast<uint32_t>(c.objv.size()), 0, state});
      }
      Run& r = c.runs.back();
      for (int j = 1; j + 1 < tk.n; j += 2) {
        const int32_t row = find_row(tk.t[j]);
        if (row == kUnknownRow) return c.error.fail(p, "unknown row '" + std::string(tk.t[j]) + "'");
        double v;
        if (!parse_number(tk.t[j + 1], &v)) {
          return c.error.fail(p, "invalid number '" + std::string(tk.t[j + 1]) + "'");
        }
        if (row == kObjectiveRow) {
          c.objv.push_back(v);
          ++r.no;
        } else if (row >= 0) {
          if (v == 0.0 || (r.ne > 0 && row <= c.rows.back())) c.clean = false;
          c.rows.push_back(row);
          c.vals.push_back(v);
          ++r.ne;
        }
      }
      return true;
    });
    c.end_state = state;
  }

  void columns(const char* b, const char* e) {
    const int parts = parts_for(static_cast<size_t>(e - b));
    const std::vector<const char*> cut = split_columns(b, e, parts);
    auto sec = std::make_unique<std::vector<ColChunk>>(static_cast<size_t>(parts));
    std::vector<ColChunk>& ch = *sec;
    run_threads(parts, [&](int t) { parse_columns(cut[t], cut[t + 1], ch[t]); });
    rethrow_first(ch);
    clock_.mark("col parse");

    // Candidates (runs) numbered in file order after those of earlier COLUMNS sections.
    const size_t base = col_keys_.size();
    std::vector<size_t> cbase(static_cast<size_t>(parts) + 1);
    cbase[0] = base;
    for (int t = 0; t < parts; ++t) cbase[t + 1] = cbase[t] + ch[t].runs.size();
    const size_t total = cbase[parts];
    if (total > static_cast<size_t>(kMaxIndex)) fail(nullptr, "too many columns", MpsStatus::kTooLarge);
    col_keys_.resize(total);
    cand_col_.resize(total);
    col_lost_.resize(total);
    run_threads(parts, [&](int t) {
      std::copy(ch[t].keys.begin(), ch[t].keys.end(), col_keys_.begin() + static_cast<std::ptrdiff_t>(cbase[t]));
      std::fill(col_lost_.begin() + static_cast<std::ptrdiff_t>(cbase[t]),
                col_lost_.begin() + static_cast<std::ptrdiff_t>(cbase[t + 1]), uint8_t{0});
    });

    // The integer-marker state at each range's start (markers persist across sections).
    std::vector<int8_t> start(static_cast<size_t>(parts));
    int8_t st = in_integer_block_;
    for (int t = 0; t < parts; ++t) {
      start[t] = st;
      if (ch[t].end_state >= 0) st = ch[t].end_state;
    }
    in_integer_block_ = st;

    col_table_.insert_range(col_keys_, base, total, col_lost_.data(), threads_for(total - base));

    // First occurrences become columns, in file order (mps_reader.cpp:265-279).
    std::vector<int64_t> wbase(static_cast<size_t>(parts) + 1, 0);
    run_threads(parts, [&](int t) {
      int64_t w = 0;
      for (size_t c = cbase[t]; c < cbase[t + 1]; ++c) w += col_lost_[c] ? 0 : 1;
      wbase[t + 1] = w;
    });
    for (int t = 0; t < parts; ++t) wbase[t + 1] += wbase[t];
    const int64_t added = wbase[parts];
    const bool repeats = added != static_cast<int64_t>(total - base);
    if (n_ + added > kMaxIndex) fail(nullptr, "more than 2^31 - 1 columns", MpsStatus::kTooLarge);
    const size_t n_new = static_cast<size_t>(n_ + added);
    col_integer_.resize(n_new);
    col_lower_.resize(n_new);
    col_upper_.resize(n_new);
    lower_set_.resize(n_new);
    col_place_.resize(n_new);
    col_cand_.resize(n_new);
    const uint32_t chunk0 = static_cast<uint32_t>(chunks_.size());
    run_threads(parts, [&](int t) {
      int32_t col = static_cast<int32_t>(n_ + wbase[t]);
      const ColChunk& c = ch[t];
      for (size_t r = 0; r < c.runs.size(); ++r) {
        const size_t cand = cbase[t] + r;
        if (col_lost_[cand]) continue;
        cand_col_[cand] = col;
        col_cand_[col] = static_cast<int32_t>(cand);
        col_place_[col] = Place{chunk0 + static_cast<uint32_t>(t), static_cast<uint32_t>(r)};
        const int8_t s = c.runs[r].state < 0 ? start[t] : c.runs[r].state;
        col_integer_[col] = static_cast<uint8_t>(s > 0);
        col_lower_[col] = 0.0;
        col_upper_[col] = kInf;
        lower_set_[col] = 0;
        ++col;
      }
    });
    // Later occurrences add to the column of the first (rare: sequential).
    if (repeats) {
      for (int t = 0; t < parts; ++t) {
        for (size_t r = 0; r < ch[t].runs.size(); ++r) {
          const size_t cand = cbase[t] + r;
          if (!col_lost_[cand]) continue;
          const int32_t owner = col_table_.find(col_keys_.data(), col_keys_[cand]);
          cand_col_[cand] = cand_col_[owner];
          extras_.push_back(Extra{cand_col_[cand], Place{chunk0 + static_cast<uint32_t>(t), static_cast<uint32_t>(r)}});
        }
      }
    }
    n_ = static_cast<int32_t>(n_new);
    for (ColChunk& c : ch) chunks_.push_back(&c);
    sections_.push_back(std::move(sec));
    clock_.mark("col table");
  }

  // ---- RHS and RANGES (mps_reader.cpp:304-344) ----
  void rhs(const char* b, const char* e, bool is_range) {
    struct Rec {
      int32_t row;
      double v;
    };
    struct Chunk {
      std::vector<Rec> recs;
      ChunkError error;
    };
    const int parts = parts_for(static_cast<size_t>(e - b));
    const std::vector<const char*> cut = split_lines(b, e, parts);
    std::vector<Chunk> ch(static_cast<size_t>(parts));
    run_threads(parts, [&](int t) {
      Chunk& c = ch[t];
      Tokens tk;
      int32_t last = -2;
      for_lines(cut[t], cut[t + 1], [&](const char* p, const char* q) {
        if (p == q || *p == '*') return true;
        tokens(p, q, tk);
        if (tk.n == 0) return true;
        const int first = tk.n % 2 == 1 ? 1 : 0;
        if (tk.n - first != 2 && tk.n - first != 4) {
          return c.error.fail(p, is_range ? "RANGES entry has the wrong number of fields"
                                          : "RHS entry has the wrong number of fields");
        }
        for (int j = first; j + 1 < tk.n; j += 2) {
          const int32_t row = find_row_after(tk.t[j], &last);
          if (row == kUnknownRow) return c.error.fail(p, "unknown row '" + std::string(tk.t[j]) + "'");
          double v;
          if (!parse_number(tk.t[j + 1], &v)) {
            return c.error.fail(p, "invalid number '" + std::string(tk.t[j + 1]) + "'");
          }
          if (is_range) {
            if (row < 0) return c.error.fail(p, "RANGES entry on an objective or free row");
            c.recs.push_back(Rec{row, v});
          } else if (row != kFreeRow) {
            c.recs.push_back(Rec{row, v});
          }
        }
        return true;
      });
    });
    rethrow_first(ch);
    if (rhs_.size() < static_cast<size_t>(m_)) {
      rhs_.resize(static_cast<size_t>(m_), 0.0);
      range_.resize(static_cast<size_t>(m_), 0.0);
      has_range_.resize(static_cast<size_t>(m_), 0);
    }
    for (const Chunk& c : ch) {
      for (const Rec& r : c.recs) {
        if (is_range) {
          range_[r.row] = r.v;
          has_range_[r.row] = 1;
        } else if (r.row == kObjectiveRow) {
          obj_offset_ = -r.v;
        } else {
          rhs_[r.row] = r.v;
        }
      }
    }
  }

  // ---- BOUNDS (mps_reader.cpp:346-400) ----
  void bounds(const char* b, const char* e) {
    struct Rec {
      int32_t col;
      uint8_t type;
      double v;
    };
    struct Chunk {
      std::vector<Rec> recs;
      ChunkError error;
    };
    const int parts = parts_for(static_cast<size_t>(e - b));
    const std::vector<const char*> cut = split_lines(b, e, parts);
    std::vector<Chunk> ch(static_cast<size_t>(parts));
    run_threads(parts, [&](int t) {
      Chunk& c = ch[t];
      Tokens tk;
      int32_t last = -2;
      for_lines(cut[t], cut[t + 1], [&](const char* p, const char* q) {
        if (p == q || *p == '*') return true;
        tokens(p, q, tk);
        if (tk.n == 0) return true;
        if (tk.n < 2) return c.error.fail(p, "BOUNDS entry is too short");
        const string_view type = tk.t[0];
        const bool no_value = iequals(type, "FR") || iequals(type, "MI") || iequals(type, "PL") ||
                              iequals(type, "BV");
        int pos = 1;  // TYPE [set] COLUMN [value]
        if (!no_value) {
          if (tk.n == 4) {
            pos = 2;
          } else if (tk.n != 3) {
            return c.error.fail(p, "BOUNDS entry has the wrong number of fields");
          }
        } else if (tk.n == 4) {
          pos = 2;
        } else if (tk.n == 3 && find_col(tk.t[2]) >= 0) {
          pos = 2;
        } else if (tk.n > 4) {
          return c.error.fail(p, "BOUNDS entry has the wrong number of fields");
        }
        const int32_t col = find_col_after(tk.t[pos], &last);
        if (col < 0) return c.error.fail(p, "unknown column '" + std::string(tk.t[pos]) + "'");
        double v = 0.0;
        if (!no_value && !parse_number(tk.t[pos + 1], &v)) {
          return c.error.fail(p, "invalid number '" + std::string(tk.t[pos + 1]) + "'");
        }
        uint8_t code;
        if (iequals(type, "UP")) {
          code = kUP;
        } else if (iequals(type, "UI")) {
          code = kUI;
        } else if (iequals(type, "LO")) {
          code = kLO;
        } else if (iequals(type, "LI")) {
          code = kLI;
        } else if (iequals(type, "FX")) {
          code = kFX;
        } else if (iequals(type, "FR")) {
          code = kFR;
        } else if (iequals(type, "MI")) {
          code = kMI;
        } else if (iequals(type, "PL")) {
          code = kPL;
        } else if (iequals(type, "BV")) {
          code = kBV;
        } else if (iequals(type, "SC")) {
          return c.error.fail(p, "semi-continuous bounds (SC) are not supported");
        } else {
          return c.error.fail(p, "unknown bound type '" + std::string(type) + "'");
        }
        c.recs.push_back(Rec{col, code, v});
        return true;
      });
    });
    rethrow_first(ch);
    for (const Chunk& c : ch) {
      for (const Rec& r : c.recs) {
        double& lower = col_lower_[r.col];
        double& upper = col_upper_[r.col];
        switch (r.type) {
          case kUP:
          case kUI:
            upper = r.v;
            if (r.v < 0.0 && lower == 0.0 && !lower_set_[r.col]) lower = -kInf;
            if (r.type == kUI) col_integer_[r.col] = 1;
            break;
          case kLO:
          case kLI:
            lower = r.v;
            lower_set_[r.col] = 1;
            if (r.type == kLI) col_integer_[r.col] = 1;
            break;
          case kFX:
            lower = upper = r.v;
            lower_set_[r.col] = 1;
            break;
          case kFR:
            lower = -kInf;
            upper = kInf;
            lower_set_[r.col] = 1;
            break;
          case kMI:
            lower = -kInf;
            lower_set_[r.col] = 1;
            break;
          case kPL: upper = kInf; break;
          case kBV:
            lower = 0.0;
            upper = 1.0;
            lower_set_[r.col] = 1;
            col_integer_[r.col] = 1;
            break;
          default: break;
        }
      }
    }
  }

  // ---- the model (mps_reader.cpp:440-484; Model::validate) ----

  // Sorts a column's entries by row (stably), adds equal rows in that order starting from 0.0
  // and drops exact zeros, in place; returns the count kept.
  static int64_t sort_merge(int32_t* r, double* v, int64_t n,
                            std::vector<std::pair<int32_t, double>>& tmp) {
    bool sorted = true;
    for (int64_t i = 1; i < n; ++i) {
      if (r[i] < r[i - 1]) {
        sorted = false;
        break;
      }
    }
    if (!sorted) {
      if (n <= 32) {
        for (int64_t i = 1; i < n; ++i) {
          const int32_t ri = r[i];
          const double vi = v[i];
          int64_t j = i;
          for (; j > 0 && r[j - 1] > ri; --j) {
            r[j] = r[j - 1];
            v[j] = v[j - 1];
          }
          r[j] = ri;
          v[j] = vi;
        }
      } else {
        tmp.resize(static_cast<size_t>(n));
        for (int64_t i = 0; i < n; ++i) tmp[i] = {r[i], v[i]};
        std::stable_sort(tmp.begin(), tmp.end(),
                         [](const auto& a, const auto& b) { return a.first < b.first; });
        for (int64_t i = 0; i < n; ++i) {
          r[i] = tmp[i].first;
          v[i] = tmp[i].second;
        }
      }
    }
    int64_t w = 0;
    for (int64_t i = 0; i < n;) {
      const int32_t row = r[i];
      double s = 0.0;
      while (i < n && r[i] == row) s += v[i++];
      if (s != 0.0) {
        r[w] = row;
        v[w] = s;
        ++w;
      }
    }
    return w;
  }

  // The CSC arrays and the objective: pass 1 sorts and merges each column where its run lies (or
  // gathers a repeated column's runs into the thread's side buffer) and counts; pass 2 copies to
  // the prefix-summed starts. Non-finite objective coefficients and entries are found on the way
  // (first objective column, in column order; any entry).
  void build_matrix(MpsModel* out, int64_t* bad_obj, bool* bad_entry) {
    const size_t n = static_cast<size_t>(n_);
    const bool repeats = !extras_.empty();
    if (!repeats && std::all_of(chunks_.begin(), chunks_.end(),
                                [](const ColChunk* c) { return c->clean; })) {
      copy_clean_ranges(out, bad_obj, bad_entry);
      return;
    }
    // Later occurrences of a column, grouped by column in file order.
    std::vector<int64_t> xptr;
    std::vector<Place> xplace;
    if (repeats) {
      xptr.assign(n + 1, 0);
      xplace.resize(extras_.size());
      for (const Extra& x : extras_) ++xptr[static_cast<size_t>(x.col) + 1];
      for (size_t j = 0; j < n; ++j) xptr[j + 1] += xptr[j];
      std::vector<int64_t> next(xptr.begin(), xptr.end() - 1);
      for (const Extra& x : extras_) xplace[static_cast<size_t>(next[x.col]++)] = x.place;
    }
    out->obj.resize(n);
    Buffer<int64_t> count(n);
    const int parts = threads_for(n + total_entries());
    struct Side {
      std::vector<int32_t> rows;
      std::vector<double> vals;
      std::vector<std::pair<int32_t, double>> tmp;
      std::vector<int64_t> at;  // per repeated column of the range: its start in rows / vals
      int64_t total = 0;
      int64_t bad_obj = -1;
      bool bad_entry = false;
    };
    std::vector<Side> side(static_cast<size_t>(parts));
    run_threads(parts, [&](int t) {
      Side& s = side[t];
      int64_t total = 0;
      for (size_t j = n * t / parts, e = n * (t + 1) / parts; j < e; ++j) {
        const Place pl = col_place_[j];
        ColChunk& c = *chunks_[pl.chunk];
        const Run& r = c.runs[pl.run];
        double o = 0.0;
        for (uint32_t k = 0; k < r.no; ++k) o += c.objv[r.o0 + k];
        const double* kept;
        if (!repeats || xptr[j] == xptr[j + 1]) {
          count[j] = sort_merge(c.rows.data() + r.e0, c.vals.data() + r.e0, r.ne, s.tmp);
          kept = c.vals.data() + r.e0;
        } else {
          const int64_t at = static_cast<int64_t>(s.rows.size());
          s.rows.insert(s.rows.end(), c.rows.begin() + r.e0, c.rows.begin() + r.e0 + r.ne);
          s.vals.insert(s.vals.end(), c.vals.begin() + r.e0, c.vals.begin() + r.e0 + r.ne);
          for (int64_t x = xptr[j]; x < xptr[j + 1]; ++x) {
            ColChunk& cx = *chunks_[xplace[x].chunk];
            const Run& rx = cx.runs[xplace[x].run];
            for (uint32_t k = 0; k < rx.no; ++k) o += cx.objv[rx.o0 + k];
            s.rows.insert(s.rows.end(), cx.rows.begin() + rx.e0, cx.rows.begin() + rx.e0 + rx.ne);
            s.vals.insert(s.vals.end(), cx.vals.begin() + rx.e0, cx.vals.begin() + rx.e0 + rx.ne);
          }
          const int64_t len = static_cast<int64_t>(s.rows.size()) - at;
          count[j] = sort_merge(s.rows.data() + at, s.vals.data() + at, len, s.tmp);
          s.rows.resize(static_cast<size_t>(at + count[j]));
          s.vals.resize(static_cast<size_t>(at + count[j]));
          s.at.push_back(at);
          kept = s.vals.data() + at;
        }
        for (int64_t k = 0; k < count[j]; ++k) s.bad_entry |= !std::isfinite(kept[k]);
        if (s.bad_obj < 0 && !std::isfinite(o)) s.bad_obj = static_cast<int64_t>(j);
        out->obj[j] = o;
        total += count[j];
      }
      s.total = total;
    });
    std::vector<int64_t> tbase(static_cast<size_t>(parts) + 1, 0);
    *bad_obj = -1;
    *bad_entry = false;
    for (int t = 0; t < parts; ++t) {
      tbase[t + 1] = tbase[t] + side[t].total;
      if (*bad_obj < 0) *bad_obj = side[t].bad_obj;
      *bad_entry = *bad_entry || side[t].bad_entry;
    }
    const int64_t nnz = tbase[parts];
    out->colptr.resize(n + 1);
    out->rowidx.resize(static_cast<size_t>(nnz));
    out->vals.resize(static_cast<size_t>(nnz));
    out->colptr[0] = 0;
    run_threads(parts, [&](int t) {
      const Side& s = side[t];
      int64_t p = tbase[t];
      size_t xi = 0;
      for (size_t j = n * t / parts, e = n * (t + 1) / parts; j < e; ++j) {
        const int64_t k = count[j];
        const int32_t* rs;
        const double* vs;
        if (!repeats || xptr[j] == xptr[j + 1]) {
          const Place pl = col_place_[j];
          const ColChunk& c = *chunks_[pl.chunk];
          rs = c.rows.data() + c.runs[pl.run].e0;
          vs = c.vals.data() + c.runs[pl.run].e0;
        } else {
          rs = s.rows.data() + s.at[xi];
          vs = s.vals.data() + s.at[xi];
          ++xi;
        }
        for (int64_t q = 0; q < k; ++q) {
          out->rowidx[static_cast<size_t>(p + q)] = rs[q];
          out->vals[static_cast<size_t>(p + q)] = vs[q];
        }
        p += k;
        out->colptr[j + 1] = p;
      }
    });
  }

  // Every column is one run of one range, its rows increasing and no value zero: the matrix is
  // the ranges' arrays end to end (columns in range order), copied one range per thread.
  void copy_clean_ranges(MpsModel* out, int64_t* bad_obj, bool* bad_entry) {
    const size_t n = static_cast<size_t>(n_), nc = chunks_.size();
    std::vector<int64_t> colb(nc + 1, 0), nzb(nc + 1, 0);
    for (size_t k = 0; k < nc; ++k) {
      colb[k + 1] = colb[k] + static_cast<int64_t>(chunks_[k]->runs.size());
      nzb[k + 1] = nzb[k] + static_cast<int64_t>(chunks_[k]->rows.size());
    }
    out->obj.resize(n);
    out->colptr.resize(n + 1);
    out->rowidx.resize(static_cast<size_t>(nzb[nc]));
    out->vals.resize(static_cast<size_t>(nzb[nc]));
    out->colptr[0] = 0;
    std::vector<int64_t> bad(nc, -1);
    std::vector<uint8_t> bade(nc, 0);
    const int parts = static_cast<int>(std::max<size_t>(1, std::min<size_t>(nc, threads_for(n + static_cast<size_t>(nzb[nc])))));
    run_threads(parts, [&](int t) {
      for (size_t k = nc * t / parts, ke = nc * (t + 1) / parts; k < ke; ++k) {
        const ColChunk& c = *chunks_[k];
        for (size_t r = 0; r < c.runs.size(); ++r) {
          const Run& run = c.runs[r];
          const size_t j = static_cast<size_t>(colb[k]) + r;
          double o = 0.0;
          for (uint32_t q = 0; q < run.no; ++q) o += c.objv[run.o0 + q];
          if (bad[k] < 0 && !std::isfinite(o)) bad[k] = static_cast<int64_t>(j);
          out->obj[j] = o;
          out->colptr[j + 1] = nzb[k] + run.e0 + run.ne;
        }
        if (!c.rows.empty()) {
          std::memcpy(out->rowidx.data() + nzb[k], c.rows.data(), c.rows.size() * sizeof(int32_t));
          std::memcpy(out->vals.data() + nzb[k], c.vals.data(), c.vals.size() * sizeof(double));
        }
        bool b = false;
        for (const double v : c.vals) b |= !std::isfinite(v);
        bade[k] = b;
      }
    });
    *bad_obj = -1;
    *bad_entry = false;
    for (size_t k = 0; k < nc; ++k) {
      if (*bad_obj < 0) *bad_obj = bad[k];
      *bad_entry = *bad_entry || bade[k];
    }
  }

  size_t total_entries() const {
    size_t s = 0;
    for (const ColChunk* c : chunks_) s += c->rows.size();
    return s;
  }

  // Names of the given keys, concatenated, with their starts (two parallel passes).
  static void copy_names(const Buffer<Key>& keys, const Buffer<int32_t>& ids, Buffer<char>& chars,
                         Buffer<int64_t>& start, int threads) {
    const size_t k = ids.size();
    start.resize(k + 1);
    std::vector<int64_t> part(static_cast<size_t>(threads) + 1, 0);
    run_threads(threads, [&](int t) {
      int64_t sum = 0;
      for (size_t i = k * t / threads, e = k * (t + 1) / threads; i < e; ++i) sum += keys[ids[i]].len;
      part[t + 1] = sum;
    });
    for (int t = 0; t < threads; ++t) part[t + 1] += part[t];
    chars.resize(static_cast<size_t>(part[threads]));
    start[0] = 0;
    run_threads(threads, [&](int t) {
      int64_t p = part[t];
      for (size_t i = k * t / threads, e = k * (t + 1) / threads; i < e; ++i) {
        const Key& key = keys[ids[i]];
        if (key.len > 0) std::memcpy(chars.data() + p, key.p, key.len);
        p += key.len;
        start[i + 1] = p;
      }
    });
  }

  // The first index with a NaN bound or an infinite bound on the wrong side (Model::validate's
  // check_bounds), or -1; *what says which.
  static int64_t bad_bounds(const Buffer<double>& lower, const Buffer<double>& upper,
                            const char** what, int threads) {
    const size_t k = lower.size();
    std::vector<int64_t> first(static_cast<size_t>(threads), -1);
    std::vector<const char*> why(static_cast<size_t>(threads), nullptr);
    run_threads(threads, [&](int t) {
      for (size_t i = k * t / threads, e = k * (t + 1) / threads; i < e; ++i) {
        if (std::isnan(lower[i]) || std::isnan(upper[i])) {
          first[t] = static_cast<int64_t>(i);
          why[t] = "has a NaN bound";
          return;
        }
        if (lower[i] == kInf || upper[i] == -kInf) {
          first[t] = static_cast<int64_t>(i);
          why[t] = "has an infinite bound on the wrong side";
          return;
        }
      }
    });
    for (int t = 0; t < threads; ++t) {
      if (first[t] >= 0) {
        *what = why[t];
        return first[t];
      }
    }
    return -1;
  }

  void finish(MpsModel* out) {
    // Reported at the last line read: ENDATA's, else the text's last (mps_reader.cpp:78-89).
    if (objective_.empty() && m_ == 0 && n_ == 0) {
      fail(last_line_ != nullptr ? last_line_ : text_ + len_, "no ROWS or COLUMNS found");
    }
    const size_t m = static_cast<size_t>(m_);
    rhs_.resize(m, 0.0);
    range_.resize(m, 0.0);
    has_range_.resize(m, 0);
    out->row_lower.resize(m);
    out->row_upper.resize(m);
    const int nt = threads_for(m + static_cast<size_t>(n_));
    run_threads(nt, [&](int t) {
      for (size_t i = m * t / nt, e = m * (t + 1) / nt; i < e; ++i) {
        const double b = rhs_[i];
        double lo = -kInf, up = kInf;
        const char kind = row_kind_[i];
        if (kind == 'E') {
          lo = up = b;
        } else if (kind == 'L') {
          up = b;
        } else {
          lo = b;
        }
        if (has_range_[i]) {
          const double r = range_[i];
          const double ar = r < 0.0 ? -r : r;
          if (kind == 'E') {
            if (r >= 0.0) {
              up = b + ar;
            } else {
              lo = b - ar;
            }
          } else if (kind == 'L') {
            lo = b - ar;
          } else {
            up = b + ar;
          }
        }
        out->row_lower[i] = lo;
        out->row_upper[i] = up;
      }
    });
    int64_t bad_obj = -1;
    bool bad_entry = false;
    build_matrix(out, &bad_obj, &bad_entry);
    clock_.mark("matrix");

    if (!std::isfinite(obj_offset_)) fail(nullptr, "objective offset is not finite");
    if (bad_obj >= 0) fail(nullptr, "objective coefficient " + std::to_string(bad_obj) + " is not finite");
    if (bad_entry) fail(nullptr, "constraint matrix contains a non-finite value");
    const char* what = nullptr;
    int64_t at = bad_bounds(col_lower_, col_upper_, &what, nt);
    if (at >= 0) fail(nullptr, "column " + std::to_string(at) + " " + what);
    at = bad_bounds(out->row_lower, out->row_upper, &what, nt);
    if (at >= 0) fail(nullptr, "row " + std::to_string(at) + " " + what);

    out->name = name_;
    out->maximize = maximize_;
    out->obj_offset = obj_offset_;
    out->m = m_;
    out->n = n_;
    out->col_lower = std::move(col_lower_);
    out->col_upper = std::move(col_upper_);
    out->col_integer = std::move(col_integer_);
    copy_names(row_keys_, row_name_id_, out->row_names, out->row_name_start, nt);
    copy_names(col_keys_, col_cand_, out->col_names, out->col_name_start, nt);
    clock_.mark("names");
  }

  struct Extra {
    int32_t col;
    Place place;
  };

  const char* text_;
  size_t len_;
  bool fixed_;                        // data lines in fixed MPS (header lines are always free)
  const char* last_line_ = nullptr;  // the ENDATA line, once read
  PhaseClock clock_;
  int hw_threads_ = 1;
  int forced_ = 0;

  std::string name_;
  bool maximize_ = false;
  double obj_offset_ = 0.0;
  std::string objective_;

  // Rows: every ROWS name (N rows included) with its value (row index, kObjectiveRow, kFreeRow).
  Buffer<Key> row_keys_;
  std::vector<int32_t> row_val_;
  Buffer<uint8_t> row_lost_;
  NameTable row_table_;
  int32_t m_ = 0;
  std::vector<char> row_kind_;       // per row: 'E', 'L' or 'G'
  Buffer<int32_t> row_name_id_;      // per row: its key
  std::vector<double> rhs_, range_;
  std::vector<uint8_t> has_range_;

  // Columns: one candidate per run of lines; the first candidate of a name is the column.
  std::vector<std::unique_ptr<std::vector<ColChunk>>> sections_;
  std::vector<ColChunk*> chunks_;
  Buffer<Key> col_keys_;
  Buffer<int32_t> cand_col_;
  Buffer<uint8_t> col_lost_;
  NameTable col_table_;
  int32_t n_ = 0;
  Buffer<int32_t> col_cand_;
  Buffer<Place> col_place_;
  std::vector<Extra> extras_;
  Buffer<uint8_t> col_integer_;
  Buffer<double> col_lower_, col_upper_;
  Buffer<uint8_t> lower_set_;
  int8_t in_integer_block_ = 0;
};

}  // namespace

MpsStatus read_mps_text(const char* text, size_t len, int threads, MpsModel* out,
                        MpsError* err) {
  static const char kEmpty[1] = {0};
  if (text == nullptr) {
    text = kEmpty;
    len = 0;
  }
  try {
    // Free MPS first; where it fails, fixed MPS, and where that fails too, the free error
    // (read_mps_from_string, mps_reader.cpp:515-527).
    MpsModel model;
    try {
      Reader(text, len, threads, false).read(&model);
    } catch (const Failure& free_error) {
      if (free_error.status != MpsStatus::kParseError) throw;
      try {
        model = MpsModel();
        Reader(text, len, threads, true).read(&model);
      } catch (const Failure& fixed_error) {
        if (fixed_error.status == MpsStatus::kParseError) throw free_error;
        throw;
      }
    }
    *out = std::move(model);
    return MpsStatus::kOk;
  } catch (const Failure& f) {
    if (err != nullptr) {
      err->line = f.at != nullptr ? 1 + std::count(text, f.at, '\n') : 0;
      err->message = f.message;
    }
    return f.status;
  } catch (const std::bad_alloc&) {
    if (err != nullptr) {
      err->line = 0;
      err->message = "out of host memory";
    }
    return MpsStatus::kOutOfMemory;
  }
}

MpsStatus read_mps_file(const char* path, int threads, MpsModel* out, MpsError* err) {
  auto io_error = [&](const std::string& m) {
    if (err != nullptr) {
      err->line = 0;
      err->message = m;
    }
    return MpsStatus::kIoError;
  };
  if (path == nullptr) return io_error("no path");
  const int fd = ::open(path, O_RDONLY | O_CLOEXEC);
  if (fd < 0) return io_error("cannot open '" + std::string(path) + "'");
  struct stat st;
  if (::fstat(fd, &st) != 0 || !S_ISREG(st.st_mode)) {
    ::close(fd);
    return io_error("'" + std::string(path) + "' is not a regular file");
  }
  const size_t size = static_cast<size_t>(st.st_size);
  std::unique_ptr<char[]> buf;
  try {
    buf.reset(new char[size > 0 ? size : 1]);
  } catch (const std::bad_alloc&) {
    ::close(fd);
    if (err != nullptr) err->message = "out of host memory";
    return MpsStatus::kOutOfMemory;
  }
  // Parallel reads of equal slices (the page cache copies at several GB/s per thread).
  const unsigned hw = std::thread::hardware_concurrency();
  const int cap = std::max(1, std::min(kMaxThreads, threads > 0 ? threads : static_cast<int>(hw == 0 ? 1 : hw)));
  const int parts = static_cast<int>(std::max<size_t>(1, std::min<size_t>(cap, size >> 23)));
  std::atomic<bool> bad{false};
  try {
    run_threads(parts, [&](int t) {
      size_t off = size * t / parts;
      const size_t e = size * (t + 1) / parts;
      while (off < e && !bad) {
        const ssize_t r = ::pread(fd, buf.get() + off, e - off, static_cast<off_t>(off));
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) {
          bad = true;
          break;
        }
        off += static_cast<size_t>(r);
      }
    });
  } catch (const std::bad_alloc&) {
    bad = true;
  }
  ::close(fd);
  if (bad) return io_error("cannot read '" + std::string(path) + "'");
  return read_mps_text(buf.get(), size, threads, out, err);
}

}  // namespace sg

// Host engine of the GB300 PDLP path (see sg_engine.cuh).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <map>
#include <mutex>
#include <random>
#include <tuple>
#include <type_traits>

#include "sg_engine.cuh"
#include "sg_transpose.h"
#include "sg_refine.cuh"

namespace sg {

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

template <typename T>
void dfree(T*& p) {
  if (p != nullptr) cudaFree(p);
  p = nullptr;
}

// The power iteration's start vector, as the reference draws it (pdlp.cpp:47-51):
// std::mt19937_64(12345) through std::uniform_real_distribution<double>(-1, 1).
std::vector<double> power_start(int m) {
  std::vector<double> u(static_cast<size_t>(m));
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> dist(-1.0, 1.0);
  for (int i = 0; i < m; ++i) u[i] = dist(rng);
  return u;
}

}  // namespace

// Tiles: a row longer than tile_nnz is reduced by whole CTAs, as ceil(len / tile_nnz) segment
// tiles of its own (kind 1); rows of more than warp_min nonzeros go by up to 8 into warp-per-row
// tiles (kind 2); the other rows go consecutively into tiles of at most tile_nnz nonzeros and
// tile_rows rows, a thread per row (kind 0).
void build_tiles(const std::vector<int>& ptr, int tile_nnz, int tile_rows, int warp_min,
                 int split, std::vector<Tile>* out, int* nlong, const std::vector<char>* adj,
                 int group_pos) {
  out->clear();
  *nlong = 0;
  const int rows = static_cast<int>(ptr.size()) - 1;
  const bool grouping = adj != nullptr && group_pos > 0 &&
                        adj->size() >= static_cast<size_t>(std::max(rows, 0));
  // Rows longer than a tile are split into CTA segments (kind 1); rows of more than
  // warp_min nonzeros get a warp each, kWarpsPerTile rows per tile (kind 2) — or, with
  // split > 0, a team of the fewest warps (a power of two up to kWarpsPerTile) giving each at
  // most `split` nonzeros, kWarpsPerTile / team rows of equal team per tile.
  const int long_len = std::max(tile_nnz, warp_min);
  auto team_of = [split](int len) {
    int t = 1;
    if (split > 0) {
      while (t < kWarpsPerTile && len > static_cast<long long>(t) * split) t *= 2;
    }
    return t;
  };
  // The run of gather-neighbour rows from row q, each longer than warp_min (at most
  // kGroupRows; 0 without grouping), and its longest row.
  auto run_at = [&](int q, int* maxlen) {
    if (!grouping || ptr[q + 1] - ptr[q] <= warp_min) return 0;
    int g = 1;
    *maxlen = ptr[q + 1] - ptr[q];
    while (g < kGroupRows && q + g < rows && (*adj)[q + g - 1] &&
           ptr[q + g + 1] - ptr[q + g] > warp_min) {
      *maxlen = std::max(*maxlen, ptr[q + g + 1] - ptr[q + g]);
      ++g;
    }
    return g;
  };
  int r = 0;
  while (r < rows) {
    const int len = ptr[r + 1] - ptr[r];
    if (grouping) {
      int maxlen = 0;
      const int g = run_at(r, &maxlen);
      if (g >= 8) {
        const int nseg = (maxlen + group_pos - 1) / group_pos;
        const int lrow = nseg > 1 ? (*nlong)++ : -1;
        for (int s = 0; s < nseg; ++s) {
          Tile t{};
          t.r0 = r;
          t.r1 = r + g;
          t.k0 = s * group_pos;
          t.k1 = std::min(maxlen, (s + 1) * group_pos);
          t.kind = 3;
          t.team = 1;
          t.seg = s;
          t.nseg = nseg;
          t.lrow = lrow;
          out->push_back(t);
        }
        r += g;
        continue;
      }
    }
    if (len > warp_min && len <= long_len) {
      Tile t{};
      t.r0 = r;
      t.team = team_of(len);
      while (r < rows && r - t.r0 < kWarpsPerTile / t.team) {
        const int l = ptr[r + 1] - ptr[r];
        if (l <= warp_min || l > long_len || team_of(l) != t.team) break;
        int unused = 0;
        if (r > t.r0 && run_at(r, &unused) >= 8) break;  // a row group starts here
        ++r;
      }
      t.r1 = r;
      t.k0 = ptr[t.r0];
      t.k1 = ptr[r];
      t.kind = 2;
      t.seg = 0;
      t.nseg = 1;
      t.lrow = -1;
      out->push_back(t);
      continue;
    }
    if (len > long_len) {
      const int nseg = (len + tile_nnz - 1) / tile_nnz;
      for (int s = 0; s < nseg; ++s) {
        Tile t{};
        t.r0 = r;
        t.r1 = r + 1;
        t.k0 = ptr[r] + s * tile_nnz;
        t.k1 = std::min(ptr[r + 1], t.k0 + tile_nnz);
        t.kind = 1;
        t.team = 1;
        t.seg = s;
        t.nseg = nseg;
        t.lrow = *nlong;
        out->push_back(t);
      }
      ++*nlong;
      ++r;
      continue;
    }
    const int r0 = r;
    while (r < rows && r - r0 < tile_rows) {
      const int l = ptr[r + 1] - ptr[r];
      if (l > warp_min) break;
      if (ptr[r + 1] - ptr[r0] > tile_nnz) break;
      ++r;
    }
    Tile t{};
    t.r0 = r0;
    t.r1 = r;
    t.k0 = ptr[r0];
    t.k1 = ptr[r];
    t.kind = 0;
    t.team = 1;
    t.seg = 0;
    t.nseg = 1;
    t.lrow = -1;
    out->push_back(t);
  }
}

int device_info(int* major, int* minor, char* name, size_t len) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return kErrNoDevice;
  }
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return kErrNoDevice;
  }
  if (major) *major = prop.major;
  if (minor) *minor = prop.minor;
  if (name && len > 0) {
    strncpy(name, prop.name, len - 1);
    name[len - 1] = '\0';
  }
  // The kernels are built for sm_103a only.
  if (prop.major * 10 + prop.minor != 103) return kErrNoDevice;
  return kOk;
}

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (chunk_exec_) cudaGraphExecDestroy(chunk_exec_);
  if (chunk_graph_) cudaGraphDestroy(chunk_graph_);
  if (chunk32_exec_) cudaGraphExecDestroy(chunk32_exec_);
  if (chunk32_graph_) cudaGraphDestroy(chunk32_graph_);
  // The buffers sized by the problem live in the arena; the tile sets and the rest are their
  // own allocations.
  for (DevOp* op : {&K_, &Kt_}) {
    dfree(op->tiles);
    dfree(op->seg_part);
    dfree(op->lcount);
    dfree(op->act_rows);
    dfree(op->st_tiles);
    dfree(op->st_seg_part);
    dfree(op->st_grp_part);
    dfree(op->st_lcount);
  }
  dfree(long_terms_);
  dfree(arena_);
  if (ctl_host_) cudaFreeHost(ctl_host_);
  for (auto& e : ev_) {
    if (e) cudaEventDestroy(e);
  }
  if (stream_) cudaStreamDestroy(stream_);
}

int Engine::check(cudaError_t e, const char* what) {
  (void)what;
  if (e == cudaSuccess) return kOk;
  return e == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda;
}

#define SG_TRY(call)                        \
  do {                                      \
    const cudaError_t e_ = (call);          \
    if (e_ != cudaSuccess) {                \
      if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return e_ == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda; \
    }                                       \
  } while (0)

int Engine::create_from_device(Engine** out, const DeviceLp& d, const Options& opt,
                               std::string* err) {
  *out = nullptr;
  if (d.m < 0 || d.n < 0 || d.kptr_host.size() != static_cast<size_t>(d.m) + 1 ||
      d.tptr_host.size() != static_cast<size_t>(d.n) + 1) {
    if (err) *err = "invalid argument";
    return kErrInvalidArgument;
  }
  if (d.nnz >= static_cast<long long>(std::numeric_limits<int>::max()) ||
      static_cast<long long>(d.n) + d.m >= std::numeric_limits<int>::max()) {
    if (err) *err = "matrix too large for 32-bit offsets";
    return kErrTooLarge;
  }
  if (device_info(nullptr, nullptr, nullptr, 0) != kOk) {
    if (err) *err = "no sm_103 GPU";
    return kErrNoDevice;
  }
  Engine* e = new Engine();
  e->m_ = d.m;
  e->n_ = d.n;
  e->nnz_ = d.nnz;
  e->opt_ = opt;
  e->fp32_ = opt.precision == 1 || opt.precision == 2;
  e->switch_ = opt.precision == 2;
  e->x_bounds_uniform_ = d.x_uniform;
  e->x_lo_ = d.x_lo;
  e->x_hi_ = d.x_hi;
  e->K_.rows = d.m;
  e->K_.cols = d.n;
  e->K_.nnz = d.nnz;
  e->K_.host_ptr = d.kptr_host;
  e->Kt_.rows = d.n;
  e->Kt_.cols = d.m;
  e->Kt_.nnz = d.nnz;
  e->Kt_.host_ptr = d.tptr_host;
  std::string why;
  int rc = e->alloc_all(&why);
  if (rc != kOk) {
    if (err) *err = why;
    delete e;
    return rc;
  }
  cudaStream_t s = e->stream_;
  const size_t nb = static_cast<size_t>(d.nnz);
  const size_t nt = static_cast<size_t>(d.n) + d.m;
  auto dd = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (bytes == 0) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s);
  };
  cudaError_t ce = dd(e->K_.ptr, d.kptr, (static_cast<size_t>(d.m) + 1) * sizeof(int));
  if (ce == cudaSuccess) ce = dd(e->K_.idx, d.kidx, nb * sizeof(int));
  if (ce == cudaSuccess) ce = dd(e->K_.val_orig, d.kval, nb * sizeof(double));
  if (ce == cudaSuccess) ce = dd(e->Kt_.ptr, d.tptr, (static_cast<size_t>(d.n) + 1) * sizeof(int));
  if (ce == cudaSuccess) ce = dd(e->Kt_.idx, d.tidx, nb * sizeof(int));
  if (ce == cudaSuccess) ce = dd(e->Kt_.val_orig, d.tval, nb * sizeof(double));
  if (ce == cudaSuccess) ce = dd(e->cost_orig_, d.cost, nt * sizeof(double));
  if (ce == cudaSuccess) ce = dd(e->lower_orig_, d.lower, nt * sizeof(double));
  if (ce == cudaSuccess) ce = dd(e->upper_orig_, d.upper, nt * sizeof(double));
  std::vector<double> u0 = power_start(d.m);
  if (ce == cudaSuccess && !u0.empty()) {
    ce = cudaMemcpyAsync(e->u0_, u0.data(), u0.size() * sizeof(double), cudaMemcpyHostToDevice,
                         s);
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&e->sm_count_, cudaDevAttrMultiProcessorCount, dev);
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    if (err) *err = std::string("device copy: ") + cudaGetErrorString(ce);
    const int code = ce == cudaErrorMemoryAllocation ? kErrOutOfMemory : kErrCuda;
    delete e;
    return code;
  }
  rc = e->set_active_rows(d.row_inert, &why);
  if (rc == kOk) rc = e->find_neighbours(&why);
  if (rc == kOk) rc = e->tune_tiles(&why);
  if (rc != kOk) {
    if (err) *err = why;
    delete e;
    return rc;
  }
  *out = e;
  return kOk;
}

namespace {

// Row-length statistics of an operator: the autotuner's cache key.
struct ShapeKey {
  int rows;
  long long nnz;
  int max_len;
  long long over32, over128, over4096;
  int fp32;
  int groups;   // the row-group option (0 tuned, 1 built-in, -1 never)
  int staging;  // the segment-staging option (1 staged, -1 direct)
  bool operator<(const ShapeKey& o) const {
    return std::tie(rows, nnz, max_len, over32, over128, over4096, fp32, groups, staging) <
           std::tie(o.rows, o.nnz, o.max_len, o.over32, o.over128, o.over4096, o.fp32,
                    o.groups, o.staging);
  }
};

std::mutex g_shape_mu;
std::map<ShapeKey, TileShape> g_shape_cache;
bool g_shape_file_read = false;

// SG_TILE_CACHE names a text file that carries the tuner's choices across processes (so that a
// profiler run, whose launches cannot be timed, uses the shapes a plain run picked): one line
// per operator, the key's nine fields then the shape's seven. Read once per process, appended
// after each tuning. Call with g_shape_mu held.
void read_shape_file() {
  if (g_shape_file_read) return;
  g_shape_file_read = true;
  const char* path = std::getenv("SG_TILE_CACHE");
  if (path == nullptr || *path == '\0') return;
  FILE* f = std::fopen(path, "r");
  if (f == nullptr) return;
  ShapeKey k{};
  TileShape sh;
  while (std::fscanf(f, "%d %lld %d %lld %lld %lld %d %d %d %d %d %d %d %d %d %d", &k.rows,
                     &k.nnz, &k.max_len, &k.over32, &k.over128, &k.over4096, &k.fp32,
                     &k.groups, &k.staging, &sh.cap_nnz, &sh.cap_rows, &sh.warp_min,
                     &sh.variant, &sh.split, &sh.groups, &sh.staged) == 16) {
    if (sh.cap_nnz >= 256 && sh.cap_nnz <= 4 * kTileNnz && sh.cap_rows >= 1 &&
        sh.cap_rows <= kTileRows && sh.warp_min >= 32 && (sh.variant == 0 || sh.variant == 1) &&
        sh.split >= 0 && (sh.groups == 0 || sh.groups == 1) &&
        (sh.staged == 0 || sh.staged == 1)) {
      g_shape_cache[k] = sh;
    }
  }
  std::fclose(f);
}

void append_shape_file(const ShapeKey& k, const TileShape& sh) {
  const char* path = std::getenv("SG_TILE_CACHE");
  if (path == nullptr || *path == '\0') return;
  FILE* f = std::fopen(path, "a");
  if (f == nullptr) return;
  std::fprintf(f, "%d %lld %d %lld %lld %lld %d %d %d %d %d %d %d %d %d %d\n", k.rows, k.nnz,
               k.max_len, k.over32, k.over128, k.over4096, k.fp32, k.groups, k.staging,
               sh.cap_nnz, sh.cap_rows, sh.warp_min, sh.variant, sh.split, sh.groups, sh.staged);
  std::fclose(f);
}

ShapeKey shape_key(const DevOp& op, bool fp32, int groups, int staging) {
  // The rows the step kernel runs over (inert rows left out are empty).
  const int rows = op.act_rows != nullptr ? static_cast<int>(op.act_list.size()) : op.rows;
  ShapeKey k{rows, op.nnz, 0, 0, 0, 0, fp32 ? 1 : 0, groups, staging};
  for (int r = 0; r < op.rows; ++r) {
    const int len = op.host_ptr[r + 1] - op.host_ptr[r];
    k.max_len = std::max(k.max_len, len);
    k.over32 += len > 32;
    k.over128 += len > 128;
    k.over4096 += len > 4096;
  }
  return k;
}

}  // namespace

// The built-in rule: a power of two between 256 and kTileNnz nonzeros per tile giving each
// operator about 8 tiles per SM (small problems spread over every SM; large ones stream long
// tiles); short-row tiles of at most half that many rows (256 to kTileRows).
TileShape Engine::default_shape(const DevOp& op) const {
  const long long target = std::max<long long>(1, op.nnz / (8LL * sm_count_));
  TileShape sh;
  int cap = 256;
  while (cap < kTileNnz && cap < target) cap *= 2;
  if (opt_.tile_nnz > 0) cap = opt_.tile_nnz;
  sh.cap_nnz = cap;
  sh.cap_rows = std::min(kTileRows, std::max(256, cap / 2));
  sh.warp_min = kWarpRowMin;
  // The deep-unroll kernel variant when most nonzeros sit in rows a warp or CTAs take.
  long long in_long = 0;
  for (int r = 0; r < op.rows; ++r) {
    const int len = op.host_ptr[r + 1] - op.host_ptr[r];
    if (len > sh.warp_min) in_long += len;
  }
  sh.variant = 2 * in_long >= op.nnz && op.nnz > 0 ? 1 : 0;
  sh.split = opt_.tile_split;
  sh.groups = opt_.row_groups > 0 ? 1 : 0;
  sh.staged = opt_.segment_staging > 0 ? 1 : 0;
  return sh;
}

// The rows of K the solves iterate over: every row but the inert ones (an empty row whose
// logical has no cost and 0 within its bounds), when the option allows and some row is inert.
int Engine::set_active_rows(const std::vector<char>& inert, std::string* err) {
  if (!opt_.skip_inert_rows || inert.size() != static_cast<size_t>(m_)) return kOk;
  std::vector<int> act;
  act.reserve(static_cast<size_t>(m_));
  for (int i = 0; i < m_; ++i) {
    if (!inert[i]) act.push_back(i);
  }
  if (act.size() == static_cast<size_t>(m_)) return kOk;
  for (int i = 0; i < m_; ++i) {
    if (inert[i] && K_.host_ptr[i + 1] != K_.host_ptr[i]) {
      if (err) *err = "inert row with nonzeros";
      return kErrInternal;
    }
  }
  K_.act_list = std::move(act);
  SG_TRY(dalloc(&K_.act_rows, K_.act_list.size()));
  if (!K_.act_list.empty()) {
    SG_TRY(cudaMemcpy(K_.act_rows, K_.act_list.data(), K_.act_list.size() * sizeof(int),
                      cudaMemcpyHostToDevice));
  }
  return kOk;
}

// Positions per segment of a kind-3 row group: a multiple of the CTA's 8 x 16-position blocks
// holding about a tile's nonzeros for 32 rows.
int group_positions(int cap_nnz) {
  const int step = (kBlock / 32) * kGroupPos;
  return std::max(step, (cap_nnz / kGroupRows) / step * step);
}

// The gather neighbours among K's rows (row_neighbours_kernel), kept on the host for the tile
// partition; none: host_adj stays empty. Also marks operators whose rows all have the same
// length (their short-row tiles need no row starts).
int Engine::find_neighbours(std::string* err) {
  for (DevOp* op : {&K_, &Kt_}) {
    const std::vector<int>& p = op->host_ptr;
    int len = op->rows > 0 ? p[1] - p[0] : 0;
    for (int r = 1; len > 0 && r < op->rows; ++r) {
      if (p[r + 1] - p[r] != len) len = 0;
    }
    op->uniform_len = len;
  }
  K_.host_adj.clear();
  if (m_ < 2 || nnz_ == 0) return kOk;
  unsigned char* d = nullptr;
  SG_TRY(dalloc(&d, static_cast<size_t>(m_)));
  launch_row_neighbours(m_, K_.ptr, K_.idx, d, stream_);
  std::vector<char> adj(static_cast<size_t>(m_));
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    e = cudaMemcpyAsync(adj.data(), d, adj.size(), cudaMemcpyDeviceToHost, stream_);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  dfree(d);
  if (e != cudaSuccess) {
    if (err) *err = std::string("row neighbours: ") + cudaGetErrorString(e);
    return kErrCuda;
  }
  for (char a : adj) {
    if (a) {
      K_.host_adj = std::move(adj);
      break;
    }
  }
  return kOk;
}

// Builds an operator's tiles for a shape and uploads them (replacing earlier ones); with
// inert rows left out or row groups, also the dual steps' tile set.
int Engine::set_tiles(DevOp* op, const TileShape& shape) {
  std::string* err = nullptr;
  std::vector<Tile> tiles;
  int nlong = 0;
  build_tiles(op->host_ptr, shape.cap_nnz, shape.cap_rows, shape.warp_min, shape.split, &tiles,
              &nlong);
  const bool grouped =
      shape.groups != 0 && op == &K_ && !op->host_adj.empty() && opt_.row_groups >= 0;
  const bool staged = shape.staged != 0 && op == &K_ && opt_.segment_staging >= 0;
  const bool step_set = op->act_rows != nullptr || grouped || staged;
  std::vector<Tile> st_tiles;
  int st_nlong = 0;
  int st_groups = 0;
  int st_staged = 0;
  if (step_set) {
    // The active rows' starts: the rows left out are empty, so consecutive active rows are
    // contiguous in the nonzeros and the tiles' nonzero ranges are the operator's own. Two
    // active rows are gather neighbours when they are neighbouring rows of the operator.
    const bool sub = op->act_rows != nullptr;
    const size_t na = sub ? op->act_list.size() : static_cast<size_t>(op->rows);
    std::vector<int> vp(na + 1, 0);
    std::vector<char> vadj;
    if (grouped) vadj.assign(na, 0);
    for (size_t v = 0; v < na; ++v) {
      const int r = sub ? op->act_list[v] : static_cast<int>(v);
      vp[v] = op->host_ptr[r];
      vp[v + 1] = op->host_ptr[r + 1];
      if (grouped && v + 1 < na) {
        const int rn = sub ? op->act_list[v + 1] : r + 1;
        vadj[v] = rn == r + 1 && op->host_adj[r];
      }
    }
    build_tiles(vp, shape.cap_nnz, shape.cap_rows, shape.warp_min, shape.split, &st_tiles,
                &st_nlong, grouped ? &vadj : nullptr,
                grouped ? group_positions(shape.cap_nnz) : 0);
    for (const Tile& t : st_tiles) {
      st_groups += t.kind == 3;
      st_staged |= staged && t.kind == 1 ? 1 : 0;
    }
  }
  SG_TRY(cudaStreamSynchronize(stream_));
  dfree(op->tiles);
  dfree(op->seg_part);
  dfree(op->lcount);
  dfree(op->st_tiles);
  dfree(op->st_seg_part);
  dfree(op->st_grp_part);
  dfree(op->st_lcount);
  op->step_set = false;
  op->cap_nnz = shape.cap_nnz;
  op->cap_rows = shape.cap_rows;
  op->warp_min = shape.warp_min;
  op->variant = shape.variant;
  op->split = shape.split;
  op->groups = grouped ? 1 : 0;
  op->staged = st_staged;
  op->ntiles = static_cast<int>(tiles.size());
  op->nlong = nlong;
  SG_TRY(dalloc(&op->tiles, tiles.size()));
  if (!tiles.empty()) {
    SG_TRY(cudaMemcpyAsync(op->tiles, tiles.data(), tiles.size() * sizeof(Tile),
                           cudaMemcpyHostToDevice, stream_));
  }
  SG_TRY(dalloc(&op->seg_part, tiles.size() * kMaxVec));
  SG_TRY(dalloc(&op->lcount, std::max(nlong, 1)));
  SG_TRY(cudaMemsetAsync(op->lcount, 0, std::max(nlong, 1) * sizeof(unsigned), stream_));
  if (step_set) {
    op->st_ntiles = static_cast<int>(st_tiles.size());
    op->st_nlong = st_nlong;
    op->st_groups = st_groups;
    op->st_staged = st_staged;
    SG_TRY(dalloc(&op->st_tiles, st_tiles.size()));
    if (!st_tiles.empty()) {
      SG_TRY(cudaMemcpyAsync(op->st_tiles, st_tiles.data(), st_tiles.size() * sizeof(Tile),
                             cudaMemcpyHostToDevice, stream_));
    }
    SG_TRY(dalloc(&op->st_seg_part, st_tiles.size() * kMaxVec));
    SG_TRY(dalloc(&op->st_grp_part, st_groups > 0 ? st_tiles.size() * kGroupRows : 1));
    SG_TRY(dalloc(&op->st_lcount, std::max(st_nlong, 1)));
    SG_TRY(cudaMemsetAsync(op->st_lcount, 0, std::max(st_nlong, 1) * sizeof(unsigned),
                           stream_));
    op->step_set = true;
  }
  SG_TRY(cudaStreamSynchronize(stream_));
  return kOk;
}

// Average device milliseconds of one step kernel (the dual step on K, or the primal step on
// K'), in the precision of the solve, over `reps` launches after two warm-up launches. The
// control block is set to run (it is re-initialised by every solve's setup).
double Engine::time_step_kernel(bool dual, int reps) {
  Ctl* c = fp32_ ? ctl32_ : ctl_;
  Ctl h;
  memset(&h, 0, sizeof(h));
  h.m = m_;
  h.n = n_;
  h.max_iter = std::numeric_limits<long long>::max();
  h.status = kRunning;
  h.tau = h.sigma = h.eta = 0.5;
  h.omega = 1.0;
  if (cudaMemcpy(c, &h, sizeof(Ctl), cudaMemcpyHostToDevice) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // The step kernels the solves run (classic or Halpern).
  const bool halpern = opt_.algorithm == 2;
  auto launch = [&](int j) {
    const int gk = std::max(1, std::min(K_.step_tiles(), 65535));
    const int gt = std::max(1, std::min(Kt_.ntiles, 65535));
    if (fp32_) {
      IterView<float> it = iter_view(it32_);
      if (dual) {
        if (halpern) {
          launch_halpern_dual(c, K_.step32(), it, j, gk, stream_);
        } else {
          launch_dual_step(c, K_.step32(), it, j, gk, stream_);
        }
      } else if (halpern) {
        launch_halpern_primal(c, Kt_.view32(), it, j, gt, stream_);
      } else {
        launch_primal_step(c, Kt_.view32(), it, j, gt, stream_);
      }
    } else {
      IterView<double> it = iter_view(it64_);
      if (dual) {
        if (halpern) {
          launch_halpern_dual(c, K_.step64(), it, j, gk, stream_);
        } else {
          launch_dual_step(c, K_.step64(), it, j, gk, stream_);
        }
      } else if (halpern) {
        launch_halpern_primal(c, Kt_.view64(), it, j, gt, stream_);
      } else {
        launch_primal_step(c, Kt_.view64(), it, j, gt, stream_);
      }
    }
  };
  launch(0);
  launch(1);
  cudaEventRecord(e0, stream_);
  for (int r = 0; r < reps; ++r) launch(r & 1);
  cudaEventRecord(e1, stream_);
  float ms = -1.0f;
  if (cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return ms / reps;
}

// Tile shapes of both operators. With autotuning, an operator of at least 2^18 nonzeros whose
// row-length statistics were not seen before in this process gets its step kernel timed for
// shapes around the built-in rule (half, same, twice and four times the nonzeros per tile,
// short-row tiles of half as many rows; each with both step kernel variants and each team
// split of the medium rows); the fastest (by a margin over the built-in shape) is kept and
// cached under the statistics.
int Engine::tune_tiles(std::string* err) {
  for (int which = 0; which < 2; ++which) {
    DevOp* op = which == 0 ? &K_ : &Kt_;
    const TileShape base = default_shape(*op);
    TileShape best = base;
    const bool tune = opt_.autotune && op->nnz >= (1LL << 18);
    ShapeKey key{};
    bool cached = false;
    if (tune) {
      key = shape_key(*op, fp32_, opt_.row_groups, opt_.segment_staging);
      std::lock_guard<std::mutex> lock(g_shape_mu);
      read_shape_file();
      auto it = g_shape_cache.find(key);
      if (it != g_shape_cache.end()) {
        best = it->second;
        cached = true;
      }
    }
    if (tune && !cached) {
      // Team splits of the medium rows: none, the median medium row's length and half of it
      // (rows longer than the split get 2-8 warps; only when medium rows exist).
      std::vector<int> medium;
      for (int r = 0; r < op->rows; ++r) {
        const int len = op->host_ptr[r + 1] - op->host_ptr[r];
        if (len > base.warp_min) medium.push_back(len);
      }
      std::vector<int> splits{0};
      if (!medium.empty()) {
        std::nth_element(medium.begin(), medium.begin() + medium.size() / 2, medium.end());
        const int med = medium[medium.size() / 2];
        splits.push_back(med);
        if (med / 2 > base.warp_min) splits.push_back(med / 2);
      }
      // Candidates: the built-in shape first, then (split, capacity, variant). A candidate
      // replaces the best so far only when it is at least kTuneMargin faster (the best of
      // three timed rounds each), so launch-to-launch noise keeps the built-in shape.
      std::vector<TileShape> cands{base};
      for (int split : splits) {
        for (int ci = 0; ci < 4; ++ci) {
          const int cap = (base.cap_nnz / 2) << ci;
          if (cap < 256 || cap > 4 * kTileNnz) continue;
          for (int variant = 0; variant < 2; ++variant) {
            TileShape sh = base;
            sh.cap_nnz = cap;
            sh.cap_rows = std::min(kTileRows, std::max(256, cap / 2));
            sh.variant = variant;
            sh.split = split;
            cands.push_back(sh);
          }
        }
      }
      constexpr double kTuneMargin = 0.97;
      double best_ms = -1.0;
      // With gather-neighbour rows, every candidate also with row groups. (Staged segments
      // are not a candidate: on the power-law LP's long rows they measured slower than the
      // direct loads at every capacity, 57.9 against 50.3 us in FP64.)
      if (which == 0 && !op->host_adj.empty() && opt_.row_groups == 0) {
        const size_t plain = cands.size();
        for (size_t c = 0; c < plain; ++c) {
          TileShape g = cands[c];
          g.groups = 1;
          cands.push_back(g);
        }
      }
      // Candidates that differ from the tiles in place only in the kernel variant reuse them
      // (the partition does not depend on the variant).
      bool built = false;
      TileShape in_place;
      for (const TileShape& sh : cands) {
        if (built && sh.cap_nnz == in_place.cap_nnz && sh.cap_rows == in_place.cap_rows &&
            sh.warp_min == in_place.warp_min && sh.split == in_place.split &&
            sh.groups == in_place.groups && sh.staged == in_place.staged) {
          op->variant = sh.variant;
        } else {
          const int rc = set_tiles(op, sh);
          if (rc != kOk) {
            if (err) *err = "autotune: tile upload failed";
            return rc;
          }
          built = true;
          in_place = sh;
        }
        double ms = -1.0;
        for (int round = 0; round < 3; ++round) {
          const double t = time_step_kernel(which == 0, 8);
          if (t < 0) {
            if (err) *err = std::string("autotune: ") + cudaGetErrorString(cudaGetLastError());
            return kErrCuda;
          }
          ms = ms < 0 ? t : std::min(ms, t);
        }
        if (best_ms < 0 || ms < kTuneMargin * best_ms) {
          best_ms = ms;
          best = sh;
        }
      }
      std::lock_guard<std::mutex> lock(g_shape_mu);
      g_shape_cache[key] = best;
      append_shape_file(key, best);
    }
    const int rc = set_tiles(op, best);
    if (rc != kOk) {
      if (err) *err = "tile upload failed";
      return rc;
    }
  }
  dfree(long_terms_);
  const int maxlong = std::max(std::max(std::max(K_.nlong, K_.st_nlong), Kt_.nlong), 1);
  if (dalloc(&long_terms_, static_cast<size_t>(maxlong) * kMaxSums) != cudaSuccess) {
    if (err) *err = "out of device memory";
    return kErrOutOfMemory;
  }
  // Grids: persistent CTAs for the evaluation kernels (2 per SM; 4 per SM measured no faster
  // on the transportation LP); one CTA per tile for the step kernels.
  const int eval_cap = sm_count_ * 2;
  grid_k_ = std::max(1, std::min(K_.ntiles, eval_cap));
  grid_t_ = std::max(1, std::min(Kt_.ntiles, eval_cap));
  grid_step_k_ = std::max(1, std::min(K_.step_tiles(), 65535));
  grid_full_k_ = std::max(1, std::min(K_.ntiles, 65535));
  grid_step_t_ = std::max(1, std::min(Kt_.ntiles, 65535));
  return kOk;
}

namespace {

// Lays buffers out in one allocation (256-byte aligned): a first pass with no base only sums
// the sizes, a second assigns the pointers in the same order.
struct Carver {
  char* base = nullptr;
  size_t used = 0;
  template <typename T>
  void take(T** p, size_t count) {
    used = (used + 255) & ~static_cast<size_t>(255);
    *p = base != nullptr ? reinterpret_cast<T*>(base + used) : nullptr;
    used += std::max<size_t>(count, 1) * sizeof(T);
  }
};

}  // namespace

int Engine::alloc_all(std::string* err) {
  const size_t nt = static_cast<size_t>(n_) + m_;
  const size_t m = static_cast<size_t>(m_);
  const size_t nb = static_cast<size_t>(nnz_);
  SG_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  for (auto& ev : ev_) SG_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  // The nonzero arrays carry kSegPad zeroed elements after the last nonzero: a staged segment's
  // bulk copies end at the 4-aligned position above it.
  auto layout = [&](Carver& c) {
    for (DevOp* op : {&K_, &Kt_}) {
      c.take(&op->ptr, static_cast<size_t>(op->rows) + 1);
      c.take(&op->idx, nb + kSegPad);
      c.take(&op->val, nb + kSegPad);
      c.take(&op->val_orig, nb + kSegPad);
      if (fp32_) c.take(&op->val32, nb + kSegPad);
    }
    c.take(&wait_error_, 1);
    for (double** p : {&it64_.V[0], &it64_.V[1], &it64_.Vbar, &it64_.Verg, &it64_.Vrst,
                       &it64_.cost, &it64_.lower, &it64_.upper}) {
      c.take(p, nt);
    }
    for (double** p : {&it64_.Y[0], &it64_.Y[1], &it64_.Yerg, &it64_.Yrst, &it64_.rhs}) {
      c.take(p, m);
    }
    if (fp32_) {
      for (float** p : {&it32_.V[0], &it32_.V[1], &it32_.Vbar, &it32_.Verg, &it32_.Vrst,
                        &it32_.cost, &it32_.lower, &it32_.upper}) {
        c.take(p, nt);
      }
      for (float** p : {&it32_.Y[0], &it32_.Y[1], &it32_.Yerg, &it32_.Yrst, &it32_.rhs}) {
        c.take(p, m);
      }
      for (double** p : {&cost_in_, &lower_in_, &upper_in_, &dvec_}) c.take(p, nt);
      for (double** p : {&rhs_in_, &bh_, &ones_m_}) c.take(p, m);
      c.take(&ones_n_, static_cast<size_t>(n_));
      c.take(&ctl32_, 1);
    }
    for (double** p : {&cost_orig_, &lower_orig_, &upper_orig_, &cost_ev_, &lower_ev_,
                       &upper_ev_, &x_out_, &scratch_n_}) {
      c.take(p, nt);
    }
    for (double** p : {&rhs_ev_, &rs_, &rn_, &pu_, &u0_, &y_out_, &ray_out_}) c.take(p, m);
    for (double** p : {&cs_, &cn_, &pv_, &inv_cs_}) c.take(p, static_cast<size_t>(n_));
    c.take(&inv_rs_, m);
    c.take(&partial_, static_cast<size_t>(4096) * kMaxSums);
    c.take(&counter_, 8);
    c.take(&ctl_, 1);
  };
  {
    Carver sizing;
    layout(sizing);
    SG_TRY(cudaMalloc(reinterpret_cast<void**>(&arena_), sizing.used));
    arena_bytes_ = sizing.used;
    Carver carve;
    carve.base = arena_;
    layout(carve);
  }
  for (DevOp* op : {&K_, &Kt_}) {
    SG_TRY(cudaMemsetAsync(op->idx + nb, 0, kSegPad * sizeof(int), stream_));
    SG_TRY(cudaMemsetAsync(op->val + nb, 0, kSegPad * sizeof(double), stream_));
    SG_TRY(cudaMemsetAsync(op->val_orig + nb, 0, kSegPad * sizeof(double), stream_));
    if (fp32_) SG_TRY(cudaMemsetAsync(op->val32 + nb, 0, kSegPad * sizeof(float), stream_));
  }
  SG_TRY(cudaMemsetAsync(wait_error_, 0, sizeof(int), stream_));
  K_.wait_error = wait_error_;
  Kt_.wait_error = wait_error_;
  if (fp32_) {
    std::vector<double> ones(std::max<size_t>(std::max<size_t>(m, n_), 1), 1.0);
    SG_TRY(cudaMemcpy(ones_n_, ones.data(), static_cast<size_t>(n_) * sizeof(double),
                      cudaMemcpyHostToDevice));
    SG_TRY(cudaMemcpy(ones_m_, ones.data(), m * sizeof(double), cudaMemcpyHostToDevice));
    SG_TRY(cudaMemsetAsync(ctl32_, 0, sizeof(Ctl), stream_));
    configure_refine_kernels();
  }
  SG_TRY(cudaMemsetAsync(counter_, 0, 8 * sizeof(unsigned), stream_));
  SG_TRY(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), stream_));
  SG_TRY(cudaHostAlloc(reinterpret_cast<void**>(&ctl_host_), sizeof(Ctl), cudaHostAllocDefault));
  memset(ctl_host_, 0, sizeof(Ctl));
  configure_kernels();
  return kOk;
}

template <typename T>
IterView<T> Engine::iter_view(DevIter<T>& it) {
  IterView<T> v;
  v.V[0] = it.V[0];
  v.V[1] = it.V[1];
  v.Vbar = it.Vbar;
  v.Y[0] = it.Y[0];
  v.Y[1] = it.Y[1];
  v.Verg = it.Verg;
  v.Yerg = it.Yerg;
  v.Vrst = it.Vrst;
  v.Yrst = it.Yrst;
  v.cost = it.cost;
  v.lower = it.lower;
  v.upper = it.upper;
  v.rhs = nullptr;
  v.n = n_;
  v.m = m_;
  // The shared column bounds hold for the problem itself (FP64 iterates, and the FP32 phase of
  // the precision switch), not for the refinement's correction problems in the FP32 buffers.
  v.xb_uniform = x_bounds_uniform_ && (std::is_same<T, double>::value || switch_) ? 1 : 0;
  v.xb_lo = static_cast<T>(x_lo_);
  v.xb_hi = static_cast<T>(x_hi_);
  return v;
}

EvalView Engine::eval_view() const {
  EvalView ev;
  ev.cs = cs_;
  ev.rs = rs_;
  ev.inv_cs = inv_cs_;
  ev.inv_rs = inv_rs_;
  ev.cost = cost_ev_;
  ev.lower = lower_ev_;
  ev.upper = upper_ev_;
  ev.rhs = nullptr;
  return ev;
}

RedView Engine::red_view() const {
  RedView r;
  r.partial = partial_;
  r.counter = counter_;
  r.long_terms = long_terms_;
  return r;
}

// Device setup (pdlp.cpp:260-316, 377-394, 490-492): working values from the originals,
// residual-scale constants, Ruiz, A_eq, scaled vectors, operator norm and step sizes; iterates
// zeroed. Asynchronous on the engine's stream.
int Engine::setup_device(const double* rhs_orig) {
  (void)rhs_orig;
  cudaStream_t s = stream_;
  const size_t nt = static_cast<size_t>(n_) + m_;
  const size_t nb = static_cast<size_t>(nnz_);
  std::string* err = nullptr;
  if (nb > 0) {
    SG_TRY(cudaMemcpyAsync(K_.val, K_.val_orig, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SG_TRY(cudaMemcpyAsync(Kt_.val, Kt_.val_orig, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  SG_TRY(cudaMemcpyAsync(cost_ev_, cost_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SG_TRY(cudaMemcpyAsync(lower_ev_, lower_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SG_TRY(cudaMemcpyAsync(upper_ev_, upper_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SG_TRY(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), s));
  // Constant fields of the control block.
  Ctl h;
  memset(&h, 0, sizeof(h));
  h.m = m_;
  h.n = n_;
  h.tol = opt_.tol;
  long long max_iter = opt_.max_iterations;
  if (max_iter <= 0) {
    // pdlp.cpp:365-373.
    max_iter = std::max<long long>(10000LL, 10000LL * (static_cast<long long>(m_) + n_) / 10);
    if (!(opt_.time_limit > 0)) max_iter = std::min<long long>(max_iter, 1000000LL);
  }
  h.max_iter = max_iter;
  h.kkt_at_restart = INFINITY;
  h.kkt_previous = INFINITY;
  h.status = kRunning;
  h.omega = 1.0;
  // Halpern: no infeasibility / unboundedness checks (they read differences of consecutive
  // PDHG iterates, which the Halpern iterates are not).
  h.halpern = opt_.algorithm == 2 ? 1 : 0;
  h.no_detect = h.halpern;
  // The reference's artificial-restart fraction for its own algorithm; the engine's algorithms
  // restart more often (0.1): on the 1M x 2M power-law LP the primal weight otherwise sits for
  // hundreds of thousands of iterations at a value 1000x too small (FP64 Halpern: 1e-8 in 52 s
  // at 0.1, relative primal residual 2.5e-6 after 60 s at 0.36), and the transportation LP
  // takes 1,984 instead of 2,112 FP64 iterations.
  h.art_frac = opt_.artificial_restart > 0 ? opt_.artificial_restart
                                           : (opt_.algorithm == 0 ? 0.36 : 0.1);
  SG_TRY(cudaMemcpyAsync(ctl_, &h, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  SG_TRY(cudaStreamSynchronize(s));  // h lives on this stack frame
  const OpView<double> K = K_.view64();
  const OpView<double> Kt = Kt_.view64();
  const RedView red = red_view();
  // Scale factors start at 1.
  {
    std::vector<double> ones(std::max(nt, static_cast<size_t>(1)), 1.0);
    SG_TRY(cudaMemcpyAsync(cs_, ones.data(), static_cast<size_t>(n_) * sizeof(double),
                           cudaMemcpyHostToDevice, s));
    SG_TRY(cudaMemcpyAsync(rs_, ones.data(), static_cast<size_t>(m_) * sizeof(double),
                           cudaMemcpyHostToDevice, s));
    SG_TRY(cudaStreamSynchronize(s));
  }
  launch_setup_norms(ctl_, K, Kt, cost_orig_, red, grid_k_, grid_t_, s);
  if (m_ > 0 && n_ > 0) {
    if (opt_.algorithm >= 1) {
      launch_enhanced_scaling(K, Kt, rs_, cs_, rn_, cn_, grid_k_, grid_t_, s);
    } else {
      for (int pass = 0; pass < 10; ++pass) {
        launch_ruiz_pass(ctl_, K, Kt, rs_, cs_, rn_, cn_, red, grid_k_, grid_t_, s);
      }
    }
  }
  launch_apply_scaling(K, Kt, rs_, cs_, nnz_, s);
  launch_reciprocals(cs_, inv_cs_, n_, s);
  launch_reciprocals(rs_, inv_rs_, m_, s);
  launch_scale_vectors(n_, m_, cs_, rs_, cost_orig_, lower_orig_, upper_orig_, nullptr,
                       it64_.cost, it64_.lower, it64_.upper, nullptr, s);
  if (m_ > 0) {
    SG_TRY(cudaMemcpyAsync(pu_, u0_, static_cast<size_t>(m_) * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
  }
  launch_power_iteration(ctl_, K, Kt, pu_, pv_, red, 20, grid_k_, grid_t_, s);
  if (opt_.algorithm >= 1) {
    launch_primal_weight_init(ctl_, n_, m_, it64_.cost, it64_.lower, it64_.upper, red, s);
  }
  // Iterates start at zero (pdlp.cpp:323-329).
  for (double* p : {it64_.V[0], it64_.V[1], it64_.Vbar, it64_.Verg, it64_.Vrst}) {
    SG_TRY(cudaMemsetAsync(p, 0, nt * sizeof(double), s));
  }
  for (double* p : {it64_.Y[0], it64_.Y[1], it64_.Yerg, it64_.Yrst}) {
    SG_TRY(cudaMemsetAsync(p, 0, static_cast<size_t>(m_) * sizeof(double), s));
  }
  SG_TRY(cudaGetLastError());
  return kOk;
}

int Engine::equilibration(double* col_scale, double* row_scale, double* op_norm,
                          double* step_size) {
  std::string* err = nullptr;
  seam_mode_ = false;
  int rc = setup_device(nullptr);
  if (rc != kOk) return rc;
  SG_TRY(cudaStreamSynchronize(stream_));
  if (col_scale && n_ > 0) {
    SG_TRY(cudaMemcpy(col_scale, cs_, static_cast<size_t>(n_) * sizeof(double),
                      cudaMemcpyDeviceToHost));
  }
  if (row_scale && m_ > 0) {
    SG_TRY(cudaMemcpy(row_scale, rs_, static_cast<size_t>(m_) * sizeof(double),
                      cudaMemcpyDeviceToHost));
  }
  Ctl h;
  SG_TRY(cudaMemcpy(&h, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
  if (op_norm) *op_norm = h.op_norm;
  if (step_size) *step_size = h.eta;
  return kOk;
}

// One chunk: kCheckFrequency fused iterations, the evaluation, the decisions, restart and
// detection. Recorded once as a CUDA graph.
namespace {

// The kernels of one chunk; returns how many launches it records.
// Ks is K over the active rows (the steps), K over every row (evaluation and detection).
template <typename T>
int enqueue_chunk(Ctl* ctl, const OpView<T>& Ks, const OpView<T>& K, const OpView<T>& Kt,
                  const IterView<T>& it, const EvalView& ev, const RedView& red,
                  double* scratch_n, int gsk, int gst, int gk, int gt, bool halpern,
                  cudaStream_t s) {
  int kernels = 0;
  for (int j = 0; j < kCheckFrequency; ++j) {
    if (Ks.ts.ntiles > 0) ++kernels;
    if (Kt.ts.ntiles > 0) ++kernels;
    if (halpern) {
      launch_halpern_primal(ctl, Kt, it, j, gst, s);
      launch_halpern_dual(ctl, Ks, it, j, gsk, s);
    } else {
      launch_dual_step(ctl, Ks, it, j, gsk, s);
      launch_primal_step(ctl, Kt, it, j, gst, s);
    }
  }
  launch_eval(ctl, K, Kt, it, ev, red, gk, gt, -1, s, halpern);
  launch_decide_a(ctl, s);
  launch_detect(ctl, K, Kt, it, ev, red, scratch_n, nullptr, gk, gt, s);
  launch_decide_b(ctl, s);
  launch_restart(ctl, it, s);
  return kernels + 2 + 1 + 6 + 1 + 1;
}

}  // namespace

void Engine::enqueue_chunk_body() {
  chunk_kernels_ = enqueue_chunk(ctl_, K_.step64(), K_.view64(), Kt_.view64(),
                                 iter_view(it64_), eval_view(), red_view(), scratch_n_,
                                 grid_step_k_, grid_step_t_, grid_k_, grid_t_,
                                 opt_.algorithm == 2, stream_);
}

int Engine::capture_chunk() {
  if (chunk_exec_ != nullptr) return kOk;
  std::string* err = nullptr;
  SG_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
  enqueue_chunk_body();
  SG_TRY(cudaStreamEndCapture(stream_, &chunk_graph_));
  SG_TRY(cudaGraphInstantiate(&chunk_exec_, chunk_graph_, 0));
  return kOk;
}

// The FP32 inner solves' chunk: FP32 operators and iterates, the correction problem's
// right-hand side, evaluation in the equilibrated space (unit scales), its own control block.
int Engine::capture_chunk32() {
  if (chunk32_exec_ != nullptr) return kOk;
  std::string* err = nullptr;
  IterView<float> it = iter_view(it32_);
  it.rhs = it32_.rhs;
  SG_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
  chunk32_kernels_ = enqueue_chunk(ctl32_, K_.step32(), K_.view32(), Kt_.view32(), it,
                                   inner_eval_view(), red_view(), scratch_n_, grid_step_k_,
                                   grid_step_t_, grid_k_, grid_t_, opt_.algorithm == 2,
                                   stream_);
  SG_TRY(cudaStreamEndCapture(stream_, &chunk32_graph_));
  SG_TRY(cudaGraphInstantiate(&chunk32_exec_, chunk32_graph_, 0));
  return kOk;
}

EvalView Engine::inner_eval_view() const {
  EvalView ev;
  ev.cs = ones_n_;
  ev.rs = ones_m_;
  ev.inv_cs = ones_n_;
  ev.inv_rs = ones_m_;
  ev.cost = cost_in_;
  ev.lower = lower_in_;
  ev.upper = upper_in_;
  ev.rhs = rhs_in_;
  return ev;
}

// The FP64 point of the refinement as an iterate (current = average = the point).
IterView<double> Engine::master_view() {
  IterView<double> v = iter_view(it64_);
  v.V[1] = v.V[0];
  v.Verg = v.V[0];
  v.Y[1] = v.Y[0];
  v.Yerg = v.Y[0];
  return v;
}

// Replays a chunk graph until the device says done, keeping a few chunks in flight; the host
// only reads the control block back (an event per chunk).
int Engine::run_loop(double deadline_s, SolveInfo* info, cudaGraphExec_t exec, Ctl* ctl,
                     int kernels_per_chunk, long long max_iter) {
  std::string* err = nullptr;
  constexpr int kInflight = 3;
  int head = 0;  // oldest in flight
  int count = 0;
  long long launches = 0;
  // Every chunk advances the device's iteration counter by kCheckFrequency until the limit, so
  // a correct run needs at most this many launches; the bound keeps the host loop finite even
  // if the device never reported done.
  const long long launch_cap = max_iter / kCheckFrequency + 2 * kInflight + 4;
  for (;;) {
    if (launches >= launch_cap) break;
    while (count < kInflight) {
      const int slot = (head + count) % 4;
      SG_TRY(cudaGraphLaunch(exec, stream_));
      SG_TRY(cudaMemcpyAsync(ctl_host_, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_));
      SG_TRY(cudaEventRecord(ev_[slot], stream_));
      ++count;
      ++launches;
    }
    SG_TRY(cudaEventSynchronize(ev_[head]));
    head = (head + 1) % 4;
    --count;
    if (opt_.verbose >= 2) {
      // Trace of the last evaluation the control block holds (a later in-flight copy may have
      // overwritten the completed one: the trace is at least as recent as the chunk).
      const Ctl& h = *ctl_host_;
      printf("it %8lld restarts %5lld omega %.3e | cur p %.2e d %.2e g %+.2e | "
             "avg p %.2e d %.2e g %+.2e\n", h.t, h.restarts, h.omega, h.meas[0][0],
             h.meas[0][1], h.meas[0][2], h.meas[1][0], h.meas[1][1], h.meas[1][2]);
    }
    // The done flag of a completed copy (later copies only ever set it too).
    if (ctl_host_->done) break;
    if (deadline_s > 0 && now_s() > deadline_s) {
      // Host-side limit: let the device finish its in-flight chunks, then stop.
      break;
    }
  }
  SG_TRY(cudaStreamSynchronize(stream_));
  SG_TRY(cudaMemcpy(ctl_host_, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  info->graph_launches += launches;
  info->kernel_launches += launches * kernels_per_chunk;
  return kOk;
}

// A staged segment's bulk copy that never completed (its bounded wait gave up) makes the
// launch's sums unusable: the call reports it (and the flag is cleared).
int Engine::check_wait_error(std::string* err) {
  int flag = 0;
  if (cudaMemcpy(&flag, wait_error_, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    if (err) *err = "reading the wait flag failed";
    return kErrCuda;
  }
  if (flag == 0) return kOk;
  cudaMemset(wait_error_, 0, sizeof(int));
  if (err) *err = "a bulk copy into shared memory did not complete";
  return kErrCuda;
}

int Engine::solve(SolveInfo* info, double* x, double* y, double* dual_ray, double* primal_ray,
                  std::string* err) {
  *info = SolveInfo();
  seam_mode_ = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, stream_);
  int rc = switch_ ? solve_switched(info, x, y, dual_ray, primal_ray)
           : fp32_ ? solve_refined(info, x, y, dual_ray, primal_ray)
                   : solve_fp64(info, x, y, dual_ray, primal_ray);
  cudaEventRecord(e1, stream_);
  if (cudaEventSynchronize(e1) == cudaSuccess) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    info->device_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != kOk) {
    if (err) *err = std::string("solve failed: ") + cudaGetErrorString(cudaGetLastError());
    return rc;
  }
  return check_wait_error(err);
}

int Engine::solve_fp64(SolveInfo* info, double* x, double* y, double* dual_ray,
                       double* primal_ray) {
  const double t0 = now_s();
  int rc = setup_device(nullptr);
  if (rc != kOk) return rc;
  rc = capture_chunk();
  if (rc != kOk) return rc;
  // Deadline on the device clock (%globaltimer), checked by the decision kernel.
  if (opt_.time_limit > 0) launch_set_deadline(ctl_, opt_.time_limit - (now_s() - t0), stream_);
  const double deadline = opt_.time_limit > 0 ? t0 + opt_.time_limit : 0.0;
  const double t_setup = now_s();
  info->setup_seconds = t_setup - t0;
  rc = run_loop(deadline, info, chunk_exec_, ctl_, chunk_kernels_, max_iterations());
  if (rc != kOk) return rc;
  return finish_fp64(info, t0, 0, x, y, dual_ray, primal_ray);
}

// Status, residuals and the answer of the FP64 loop that has just ended (its control block is
// in ctl_host_); `iterations_before` iterations of an earlier phase are added to the count.
int Engine::finish_fp64(SolveInfo* info, double t0, long long iterations_before, double* x,
                        double* y, double* dual_ray, double* primal_ray) {
  std::string* err = nullptr;
  const Ctl& c = *ctl_host_;
  if (c.done == 0) {
    // The host's own time limit ended the loop.
    info->status = kTimeLimit;
    info->iterations = iterations_before + c.t;
  } else {
    info->status = c.status;
    info->iterations = iterations_before + c.iterations;
  }
  info->rel_primal = c.res[0];
  info->rel_dual = c.res[1];
  info->rel_gap = c.res[2];
  info->primal_obj = c.pobj;
  info->dual_obj = c.dobj;
  info->restarts = c.restarts;
  info->evaluations = c.evaluations;
  info->omega = c.omega;
  info->step_size = c.eta;
  info->operator_norm = c.op_norm;
  if (c.done == 0 || c.status == kTimeLimit || c.status == kIterationLimit) {
    // The relative residuals of the last evaluation's current iterate (Halpern: of T(z), the
    // only point it measures and the answer).
    const int slot = c.halpern ? 1 : 0;
    info->rel_primal = c.meas[slot][0];
    info->rel_dual = c.meas[slot][1];
    info->rel_gap = c.meas[slot][2];
  }
  // Answer.
  IterView<double> it = iter_view(it64_);
  const EvalView ev = eval_view();
  if (c.done == 0) {
    // Make the extract kernel read the current iterate.
    Ctl h = c;
    h.result_average = 0;
    SG_TRY(cudaMemcpy(ctl_, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  }
  launch_extract(ctl_, it, ev, x_out_, y_out_, c.status == kInfeasible ? ray_out_ : nullptr,
                 nullptr, stream_);
  SG_TRY(cudaGetLastError());
  const size_t nt = static_cast<size_t>(n_) + m_;
  if (x) SG_TRY(cudaMemcpyAsync(x, x_out_, nt * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  if (y && m_ > 0) {
    SG_TRY(cudaMemcpyAsync(y, y_out_, static_cast<size_t>(m_) * sizeof(double),
                           cudaMemcpyDeviceToHost, stream_));
  }
  if (c.status == kInfeasible && dual_ray && m_ > 0) {
    SG_TRY(cudaMemcpyAsync(dual_ray, ray_out_, static_cast<size_t>(m_) * sizeof(double),
                           cudaMemcpyDeviceToHost, stream_));
    info->has_dual_ray = 1;
  }
  if (c.status == kUnbounded && primal_ray && n_ > 0) {
    SG_TRY(cudaMemcpyAsync(primal_ray, scratch_n_, static_cast<size_t>(n_) * sizeof(double),
                           cudaMemcpyDeviceToHost, stream_));
    info->has_primal_ray = 1;
  }
  SG_TRY(cudaStreamSynchronize(stream_));
  info->solve_seconds = now_s() - t0;
  return kOk;
}

long long Engine::max_iterations() const {
  long long max_iter = opt_.max_iterations;
  if (max_iter <= 0) {
    // pdlp.cpp:365-373.
    max_iter = std::max<long long>(10000LL, 10000LL * (static_cast<long long>(m_) + n_) / 10);
    if (!(opt_.time_limit > 0)) max_iter = std::min<long long>(max_iter, 1000000LL);
  }
  return max_iter;
}

namespace {

// The reference's relative residuals and gap (pdlp.cpp:493-519) from the seven sums.
void finish_host(const Ctl& c, const double* s, double* rp, double* rd, double* rg) {
  const double primal_scale = 1.0 + c.a_norm_max_col * sqrt(s[4]) + sqrt(s[5]);
  const double dual_scale = 1.0 + c.at_norm_max_row * sqrt(s[6]) + c.c_norm;
  const double gap_scale = 1.0 + fabs(s[2]) + fabs(s[3]);
  *rp = c.m > 0 ? sqrt(s[0]) / primal_scale : 0.0;
  *rd = c.m > 0 ? sqrt(s[1]) / dual_scale : 0.0;
  *rg = (s[2] - s[3]) / gap_scale;
}

}  // namespace

// Device setup of the FP32 paths: the FP64 setup (equilibration, operator norm), FP32 copies
// of the equilibrated operators, the FP32 control block (the FP64 one's step size and initial
// weight, the norms of the equilibrated matrix for its relative residuals), its chunk graph.
int Engine::prepare_fp32() {
  std::string* err = nullptr;
  cudaStream_t s = stream_;
  int rc = setup_device(nullptr);
  if (rc != kOk) return rc;
  const long long nb = nnz_;
  launch_convert(K_.val, K_.val32, nb, s);
  launch_convert(Kt_.val, Kt_.val32, nb, s);
  SG_TRY(cudaMemcpyAsync(ctl32_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToDevice, s));
  launch_setup_norms(ctl32_, K_.view64(), Kt_.view64(), it64_.cost, red_view(), grid_k_, grid_t_,
                     s);
  SG_TRY(cudaStreamSynchronize(s));
  {
    Ctl h;
    SG_TRY(cudaMemcpy(&h, ctl32_, sizeof(Ctl), cudaMemcpyDeviceToHost));
    h.ir_omega0 = h.omega;
    h.q_norm = 0.0;
    SG_TRY(cudaMemcpy(ctl32_, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  }
  return capture_chunk32();
}

// The correction-problem view of the refinement kernels over the engine's buffers.
IrView Engine::ir_view() {
  IrView irv;
  irv.v = it64_.V[0];
  irv.y = it64_.Y[0];
  irv.cost_eq = it64_.cost;
  irv.lower_eq = it64_.lower;
  irv.upper_eq = it64_.upper;
  irv.bh = bh_;
  irv.d = dvec_;
  irv.cost_in = cost_in_;
  irv.lower_in = lower_in_;
  irv.upper_in = upper_in_;
  irv.rhs_in = rhs_in_;
  irv.cost32 = it32_.cost;
  irv.lower32 = it32_.lower;
  irv.upper32 = it32_.upper;
  irv.rhs32 = it32_.rhs;
  irv.red = red_view();
  irv.n = n_;
  irv.m = m_;
  return irv;
}

// Precision switch: FP32 PDLP on the equilibrated problem (FP32 operators, iterates and
// evaluation) to the inner tolerance (or until it stalls), then the same run continued in FP64:
// iterates, extrapolated point, averages, restart point, counters and primal weight carried
// over. On the transportation LP the FP64 phase then takes 1,280 iterations after 2,304 FP32
// ones; restarting the FP64 PDLP at the FP32 answer took 1,472.
// The FP32 phase does the bulk of the iterations at half the bytes and with FP32 arithmetic;
// the FP64 phase meets the reference's relative KKT test at the requested tolerance (and runs
// its infeasibility checks).
int Engine::solve_switched(SolveInfo* info, double* x, double* y, double* dual_ray,
                           double* primal_ray) {
  std::string* err = nullptr;
  const double t0 = now_s();
  cudaStream_t s = stream_;
  int rc = prepare_fp32();
  if (rc != kOk) return rc;
  rc = capture_chunk();
  if (rc != kOk) return rc;
  const size_t nt = static_cast<size_t>(n_) + m_;
  // FP32 phase: the correction problem of round 0 is the equilibrated problem itself.
  const IrView irv = ir_view();
  launch_ir_scales(ctl32_, 0, 1e4, s);
  launch_ir_build(ctl32_, irv, 0, s);
  for (float* p : {it32_.V[0], it32_.V[1], it32_.Vbar, it32_.Verg, it32_.Vrst}) {
    SG_TRY(cudaMemsetAsync(p, 0, nt * sizeof(float), s));
  }
  for (float* p : {it32_.Y[0], it32_.Y[1], it32_.Yerg, it32_.Yrst}) {
    SG_TRY(cudaMemsetAsync(p, 0, static_cast<size_t>(m_) * sizeof(float), s));
  }
  launch_norm_into(cost_in_, static_cast<long long>(nt), red_view(), &ctl32_->c_norm, s);
  launch_norm_into(rhs_in_, m_, red_view(), &ctl32_->q_norm, s);
  const long long max_iter = max_iterations();
  launch_ir_reset(ctl32_, std::max(opt_.inner_tol, opt_.tol), max_iter, kStallEvaluations, s);
  if (opt_.time_limit > 0) launch_set_deadline(ctl32_, opt_.time_limit - (now_s() - t0), s);
  const double deadline = opt_.time_limit > 0 ? t0 + opt_.time_limit : 0.0;
  info->setup_seconds = now_s() - t0;
  rc = run_loop(deadline, info, chunk32_exec_, ctl32_, chunk32_kernels_, max_iter);
  if (rc != kOk) return rc;
  const long long fp32_restarts = ctl_host_->restarts;
  const long long fp32_evals = ctl_host_->evaluations;
  // FP64 phase: the same run continued in FP64 (its iteration count includes the FP32 phase).
  IterView<float> it32 = iter_view(it32_);
  launch_continue(ctl_, ctl32_, it32, iter_view(it64_), s);
  if (opt_.time_limit > 0) launch_set_deadline(ctl_, opt_.time_limit - (now_s() - t0), s);
  rc = run_loop(deadline, info, chunk_exec_, ctl_, chunk_kernels_, max_iter);
  if (rc != kOk) return rc;
  rc = finish_fp64(info, t0, 0, x, y, dual_ray, primal_ray);
  info->restarts += fp32_restarts;
  info->evaluations += fp32_evals;
  info->refinement_rounds = 1;
  return rc;
}

// FP32 storage and arithmetic in the iterations, FP64 for the point, the residuals, the scale
// factors and every decision: round 0 solves the problem itself in FP32 to the inner
// tolerance, every later round an FP32 correction problem built from the FP64 residuals; the
// FP64 point stops when it meets the reference's relative KKT test at the requested tolerance.
int Engine::solve_refined(SolveInfo* info, double* x, double* y, double* dual_ray,
                          double* primal_ray) {
  (void)dual_ray;
  (void)primal_ray;
  std::string* err = nullptr;
  const double t0 = now_s();
  cudaStream_t s = stream_;
  int rc = prepare_fp32();
  if (rc != kOk) return rc;
  const size_t nt = static_cast<size_t>(n_) + m_;
  // The FP64 point starts at zero.
  SG_TRY(cudaMemsetAsync(it64_.V[0], 0, nt * sizeof(double), s));
  SG_TRY(cudaMemsetAsync(it64_.Y[0], 0, static_cast<size_t>(m_) * sizeof(double), s));
  SG_TRY(cudaMemsetAsync(it64_.Vrst, 0, nt * sizeof(double), s));
  SG_TRY(cudaMemsetAsync(it64_.Yrst, 0, static_cast<size_t>(m_) * sizeof(double), s));
  const IrView irv = ir_view();
  IterView<float> it32 = iter_view(it32_);
  it32.rhs = it32_.rhs;
  const IterView<double> master = master_view();
  const long long inner_max = max_iterations();
  const double deadline = opt_.time_limit > 0 ? t0 + opt_.time_limit : 0.0;
  info->setup_seconds = now_s() - t0;
  long long total_iters = 0;
  double rp = INFINITY, rd = INFINITY, rg = INFINITY, pobj = 0.0, dobj = 0.0;
  int status = kIterationLimit;
  int rounds = 0;
  // A correction round gets at most four times the first round's iterations; a round that
  // stalls hands the refined point to the FP64 PDLP (below).
  long long round0_iters = 0;
  double round0_omega = 1.0;
  bool stalled = false;
  for (int round = 0; round < opt_.refine_max_rounds; ++round) {
    long long budget = inner_max - total_iters;
    if (round > 0) {
      budget = std::min(budget, std::max<long long>(10000, 4 * round0_iters));
      launch_ir_residual(ctl32_, K_.view64(), Kt_.view64(), irv, grid_k_, grid_t_, s);
    }
    if (budget <= 0) break;
    launch_ir_scales(ctl32_, round, 1e4, s);
    launch_ir_build(ctl32_, irv, round, s);
    for (float* p : {it32_.V[0], it32_.V[1], it32_.Vbar, it32_.Verg, it32_.Vrst}) {
      SG_TRY(cudaMemsetAsync(p, 0, nt * sizeof(float), s));
    }
    for (float* p : {it32_.Y[0], it32_.Y[1], it32_.Yerg, it32_.Yrst}) {
      SG_TRY(cudaMemsetAsync(p, 0, static_cast<size_t>(m_) * sizeof(float), s));
    }
    launch_norm_into(cost_in_, static_cast<long long>(nt), red_view(), &ctl32_->c_norm, s);
    launch_norm_into(rhs_in_, m_, red_view(), &ctl32_->q_norm, s);
    launch_ir_reset(ctl32_, opt_.inner_tol, budget, kStallEvaluations, s);
    if (opt_.time_limit > 0) launch_set_deadline(ctl32_, opt_.time_limit - (now_s() - t0), s);
    rc = run_loop(deadline, info, chunk32_exec_, ctl32_, chunk32_kernels_, budget);
    if (rc != kOk) return rc;
    total_iters += ctl_host_->t;
    if (round == 0) {
      round0_iters = ctl_host_->t;
      round0_omega = ctl_host_->omega;
    } else if (ctl_host_->status != kOptimal) {
      stalled = true;
    }
    info->restarts += ctl_host_->restarts;
    info->evaluations += ctl_host_->evaluations;
    info->omega = ctl_host_->omega;
    launch_ir_update(ctl32_, it32, irv, round, s);
    // FP64 evaluation of the original problem at the refined point.
    launch_eval(ctl_, K_.view64(), Kt_.view64(), master, eval_view(), red_view(), grid_k_,
                grid_t_, 0, s);
    SG_TRY(cudaGetLastError());
    SG_TRY(cudaStreamSynchronize(s));
    Ctl h;
    SG_TRY(cudaMemcpy(&h, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
    double sums[7];
    for (int q = 0; q < 7; ++q) sums[q] = h.eval_c[q] + h.eval_r[q];
    finish_host(h, sums, &rp, &rd, &rg);
    pobj = sums[2];
    dobj = sums[3];
    rounds = round + 1;
    if (opt_.verbose) {
      printf("refine round %d: %lld inner iterations, rel primal %.3e dual %.3e gap %.3e\n",
             round, ctl_host_->t, rp, rd, rg);
    }
    if (rp < opt_.tol && rd < opt_.tol && fabs(rg) < opt_.tol) {
      status = kOptimal;
      break;
    }
    if (deadline > 0 && now_s() > deadline) {
      status = kTimeLimit;
      break;
    }
    if (stalled) break;
  }
  if (status == kIterationLimit && total_iters < inner_max) {
    // The refinement did not reach the tolerance: the FP64 PDLP continues from the refined
    // point (restarted there, with the first round's primal weight).
    rc = capture_chunk();
    if (rc != kOk) return rc;
    const long long left = inner_max - total_iters;
    launch_restart_at_point(ctl_, round0_omega, iter_view(it64_), left, s);
    if (opt_.time_limit > 0) launch_set_deadline(ctl_, opt_.time_limit - (now_s() - t0), s);
    rc = run_loop(deadline, info, chunk_exec_, ctl_, chunk_kernels_, left);
    if (rc != kOk) return rc;
    const long long restarts = info->restarts, evaluations = info->evaluations;
    rc = finish_fp64(info, t0, total_iters, x, y, dual_ray, primal_ray);
    info->restarts += restarts;
    info->evaluations += evaluations;
    info->refinement_rounds = rounds;
    return rc;
  }
  info->status = status;
  info->iterations = total_iters;
  info->refinement_rounds = rounds;
  info->rel_primal = rp;
  info->rel_dual = rd;
  info->rel_gap = rg;
  info->primal_obj = pobj;
  info->dual_obj = dobj;
  {
    Ctl h;
    SG_TRY(cudaMemcpy(&h, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
    info->step_size = h.eta;
    info->operator_norm = h.op_norm;
    h.t = 0;
    h.result_average = 0;
    SG_TRY(cudaMemcpy(ctl_, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  }
  launch_extract(ctl_, master, eval_view(), x_out_, y_out_, nullptr, nullptr, s);
  SG_TRY(cudaGetLastError());
  if (x) SG_TRY(cudaMemcpyAsync(x, x_out_, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (y && m_ > 0) {
    SG_TRY(cudaMemcpyAsync(y, y_out_, static_cast<size_t>(m_) * sizeof(double),
                           cudaMemcpyDeviceToHost, s));
  }
  SG_TRY(cudaStreamSynchronize(s));
  info->solve_seconds = now_s() - t0;
  return kOk;
}

// ---------------------------------------------------------------------------------------------
// Inner seam (the reference's gpu::PdhgDevice): here the uploaded problem is used as already
// equilibrated, and the host supplies the step sizes.

int Engine::seam_set_original(const double* cs, const double* rs, const double* cost,
                              const double* lower, const double* upper) {
  std::string* err = nullptr;
  cudaStream_t s = stream_;
  const size_t nt = static_cast<size_t>(n_) + m_;
  const size_t nb = static_cast<size_t>(nnz_);
  if (!seam_mode_) {
    // Working values = the given (equilibrated) values; vectors as given; iterates zero.
    if (nb > 0) {
      SG_TRY(cudaMemcpyAsync(K_.val, K_.val_orig, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
      SG_TRY(cudaMemcpyAsync(Kt_.val, Kt_.val_orig, nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    SG_TRY(cudaMemcpyAsync(it64_.cost, cost_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SG_TRY(cudaMemcpyAsync(it64_.lower, lower_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SG_TRY(cudaMemcpyAsync(it64_.upper, upper_orig_, nt * sizeof(double), cudaMemcpyDeviceToDevice, s));
    for (double* p : {it64_.V[0], it64_.V[1], it64_.Vbar, it64_.Verg, it64_.Vrst}) {
      SG_TRY(cudaMemsetAsync(p, 0, nt * sizeof(double), s));
    }
    for (double* p : {it64_.Y[0], it64_.Y[1], it64_.Yerg, it64_.Yrst}) {
      SG_TRY(cudaMemsetAsync(p, 0, static_cast<size_t>(m_) * sizeof(double), s));
    }
    Ctl h;
    memset(&h, 0, sizeof(h));
    h.m = m_;
    h.n = n_;
    h.max_iter = std::numeric_limits<long long>::max();
    h.status = kRunning;
    SG_TRY(cudaMemcpyAsync(ctl_, &h, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    SG_TRY(cudaStreamSynchronize(s));
    seam_mode_ = true;
    seam_fp32_ = false;
    seam_steps_ = 0;
  }
  SG_TRY(cudaMemcpyAsync(cs_, cs, static_cast<size_t>(n_) * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_TRY(cudaMemcpyAsync(rs_, rs, static_cast<size_t>(m_) * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_reciprocals(cs_, inv_cs_, n_, s);
  launch_reciprocals(rs_, inv_rs_, m_, s);
  SG_TRY(cudaMemcpyAsync(cost_ev_, cost, nt * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_TRY(cudaMemcpyAsync(lower_ev_, lower, nt * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_TRY(cudaMemcpyAsync(upper_ev_, upper, nt * sizeof(double), cudaMemcpyHostToDevice, s));
  SG_TRY(cudaStreamSynchronize(s));
  return kOk;
}

int Engine::seam_ctl_write(double tau, double sigma, long long t, long long k,
                           long long max_iter) {
  std::string* err = nullptr;
  SG_TRY(cudaStreamSynchronize(stream_));
  SG_TRY(cudaMemcpy(ctl_host_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
  ctl_host_->tau = tau;
  ctl_host_->sigma = sigma;
  ctl_host_->t = t;
  ctl_host_->k = k;
  ctl_host_->done = 0;
  ctl_host_->max_iter = max_iter;
  SG_TRY(cudaMemcpy(ctl_, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice));
  return kOk;
}

int Engine::seam_step(double tau, double sigma, long long iter) {
  std::string* err = nullptr;
  if (!seam_mode_) return kErrNotReady;
  // Step sizes and counters through the control block: t = steps taken (buffer parity),
  // k = `iter` (the averaging weight 1 / (iter + 1)).
  int rc = seam_ctl_write(tau, sigma, seam_steps_, iter, std::numeric_limits<long long>::max());
  if (rc != kOk) return rc;
  if (seam_fp32_) {
    IterView<float> it = iter_view(it32_);
    launch_dual_step(ctl_, seam_dual32(), it, 0, seam_grid_k(), stream_);
    launch_primal_step(ctl_, Kt_.view32(), it, 0, grid_step_t_, stream_);
  } else {
    IterView<double> it = iter_view(it64_);
    launch_dual_step(ctl_, seam_dual64(), it, 0, seam_grid_k(), stream_);
    launch_primal_step(ctl_, Kt_.view64(), it, 0, grid_step_t_, stream_);
  }
  SG_TRY(cudaGetLastError());
  SG_TRY(cudaStreamSynchronize(stream_));
  return kOk;
}

// One reflected Halpern iteration with the solve's kernels: the primal launch, then the dual
// launch, Halpern weight 1 / (k + 2); the iteration limit is set to this step so that the
// kernels also write T(z) into the average slots (as a chunk's last step does).
int Engine::seam_halpern_step(double tau, double sigma, long long k) {
  std::string* err = nullptr;
  if (!seam_mode_) return kErrNotReady;
  if (k < 0) return kErrInvalidArgument;
  int rc = seam_ctl_write(tau, sigma, seam_steps_, k, seam_steps_ + 1);
  if (rc != kOk) return rc;
  if (seam_fp32_) {
    IterView<float> it = iter_view(it32_);
    launch_halpern_primal(ctl_, Kt_.view32(), it, 0, grid_step_t_, stream_);
    launch_halpern_dual(ctl_, seam_dual32(), it, 0, seam_grid_k(), stream_);
  } else {
    IterView<double> it = iter_view(it64_);
    launch_halpern_primal(ctl_, Kt_.view64(), it, 0, grid_step_t_, stream_);
    launch_halpern_dual(ctl_, seam_dual64(), it, 0, seam_grid_k(), stream_);
  }
  SG_TRY(cudaGetLastError());
  SG_TRY(cudaStreamSynchronize(stream_));
  return kOk;
}

namespace {

template <typename T>
int upload_as(const double* src, T* dst, size_t count, cudaStream_t s) {
  if (count == 0) return kOk;
  std::vector<T> h(count);
  for (size_t i = 0; i < count; ++i) h[i] = static_cast<T>(src[i]);
  if (cudaMemcpyAsync(dst, h.data(), count * sizeof(T), cudaMemcpyHostToDevice, s) !=
      cudaSuccess) {
    return kErrCuda;
  }
  // The staging vector must outlive the copy.
  return cudaStreamSynchronize(s) == cudaSuccess ? kOk : kErrCuda;
}

template <typename T>
int download_as(const T* src, double* dst, size_t count) {
  if (dst == nullptr || count == 0) return kOk;
  std::vector<T> h(count);
  if (cudaMemcpy(h.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess) {
    return kErrCuda;
  }
  for (size_t i = 0; i < count; ++i) dst[i] = static_cast<double>(h[i]);
  return kOk;
}

template <typename T>
int set_iterate_state(DevIter<T>& it, int p, size_t nt, size_t m, const double* v,
                      const double* y, const double* v0, const double* y0, cudaStream_t s) {
  int rc = kOk;
  for (T* dst : {it.V[p], it.Vbar}) {
    if (rc == kOk) rc = upload_as(v, dst, nt, s);
  }
  if (rc == kOk) rc = upload_as(v0, it.Vrst, nt, s);
  if (rc == kOk) rc = upload_as(y, it.Y[p], m, s);
  if (rc == kOk) rc = upload_as(y0, it.Yrst, m, s);
  if (rc != kOk) return rc;
  if (cudaMemsetAsync(it.Verg, 0, nt * sizeof(T), s) != cudaSuccess) return kErrCuda;
  if (m > 0 && cudaMemsetAsync(it.Yerg, 0, m * sizeof(T), s) != cudaSuccess) return kErrCuda;
  return kOk;
}

}  // namespace

// The iterate the next single step starts from: current point v (n + m) and y (m) in the
// buffers of the current step parity, the extrapolated point equal to v (the reference's first
// step, v_prev = v), the anchor / restart point (v0, y0), averages zero. precision 1 uses the
// FP32 set (needs an engine created with an FP32 precision): the uploaded values, cost and
// bounds are rounded to FP32 here, and every later step, evaluation and download of the seam
// runs the FP32 kernels.
int Engine::seam_set_state(int precision, const double* v, const double* y, const double* v0,
                           const double* y0) {
  std::string* err = nullptr;
  if (!seam_mode_) return kErrNotReady;
  if (precision != 0 && !fp32_) return kErrInvalidArgument;
  if (v == nullptr || v0 == nullptr || (m_ > 0 && (y == nullptr || y0 == nullptr))) {
    return kErrInvalidArgument;
  }
  cudaStream_t s = stream_;
  const size_t nt = static_cast<size_t>(n_) + m_;
  const size_t m = static_cast<size_t>(m_);
  const int p = static_cast<int>(seam_steps_ & 1);
  SG_TRY(cudaStreamSynchronize(s));
  seam_fp32_ = precision != 0;
  int rc;
  if (seam_fp32_) {
    launch_convert(K_.val, K_.val32, nnz_, s);
    launch_convert(Kt_.val, Kt_.val32, nnz_, s);
    launch_convert(it64_.cost, it32_.cost, static_cast<long long>(nt), s);
    launch_convert(it64_.lower, it32_.lower, static_cast<long long>(nt), s);
    launch_convert(it64_.upper, it32_.upper, static_cast<long long>(nt), s);
    SG_TRY(cudaGetLastError());
    rc = set_iterate_state(it32_, p, nt, m, v, y, v0, y0, s);
  } else {
    rc = set_iterate_state(it64_, p, nt, m, v, y, v0, y0, s);
  }
  if (rc != kOk) return rc;
  SG_TRY(cudaStreamSynchronize(s));
  return kOk;
}

int Engine::seam_advance() {
  if (!seam_mode_) return kErrNotReady;
  ++seam_steps_;
  return kOk;
}

// The evaluation kernels on the seam's iterate (v_new after step()) and average: FP64 in the
// space before equilibration (the given scales and original data), FP32 in the given problem's
// own space (the FP32 evaluation of the inner solves, unit scales).
int Engine::seam_eval_launch() {
  std::string* err = nullptr;
  const int parity = static_cast<int>((seam_steps_ + 1) & 1);
  if (seam_fp32_) {
    launch_eval(ctl_, K_.view32(), Kt_.view32(), iter_view(it32_), eval_view(), red_view(),
                grid_k_, grid_t_, parity, stream_);
  } else {
    launch_eval(ctl_, K_.view64(), Kt_.view64(), iter_view(it64_), eval_view(), red_view(),
                grid_k_, grid_t_, parity, stream_);
  }
  SG_TRY(cudaGetLastError());
  SG_TRY(cudaStreamSynchronize(stream_));
  SG_TRY(cudaMemcpy(ctl_host_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
  return kOk;
}

int Engine::seam_evaluate(int which, double* sums7) {
  if (!seam_mode_) return kErrNotReady;
  const int rc = seam_eval_launch();
  if (rc != kOk) return rc;
  const int w = which == 0 ? 0 : 1;
  for (int q = 0; q < 7; ++q) sums7[q] = ctl_host_->eval_c[w * 7 + q] + ctl_host_->eval_r[w * 7 + q];
  return kOk;
}

int Engine::seam_restart_distance(int which, double* dv, double* dy) {
  if (!seam_mode_) return kErrNotReady;
  const int rc = seam_eval_launch();
  if (rc != kOk) return rc;
  const int a = which == 0 ? 14 : 16;
  *dv = ctl_host_->eval_c[a] + ctl_host_->eval_r[a];
  *dy = ctl_host_->eval_r[a + 1];
  return kOk;
}

int Engine::seam_restart_to(int which) {
  std::string* err = nullptr;
  if (!seam_mode_) return kErrNotReady;
  // The restart kernel restarts at the iterate in buffer (t & 1) or the average.
  SG_TRY(cudaStreamSynchronize(stream_));
  SG_TRY(cudaMemcpy(ctl_host_, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost));
  ctl_host_->t = seam_steps_ + 1;
  ctl_host_->restart_pending = 1;
  ctl_host_->restart_to_avg = which == 0 ? 0 : 1;
  SG_TRY(cudaMemcpy(ctl_, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice));
  if (seam_fp32_) {
    launch_restart(ctl_, iter_view(it32_), stream_);
  } else {
    launch_restart(ctl_, iter_view(it64_), stream_);
  }
  SG_TRY(cudaGetLastError());
  SG_TRY(cudaStreamSynchronize(stream_));
  ctl_host_->restart_pending = 0;
  ctl_host_->t = seam_steps_;
  SG_TRY(cudaMemcpy(ctl_, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice));
  return kOk;
}

int Engine::seam_download(double* v, double* v_new, double* y, double* y_new, double* v_erg,
                          double* y_erg) {
  std::string* err = nullptr;
  if (!seam_mode_) return kErrNotReady;
  const size_t nt = static_cast<size_t>(n_) + m_;
  const size_t m = static_cast<size_t>(m_);
  const int p = static_cast<int>(seam_steps_ & 1);
  SG_TRY(cudaStreamSynchronize(stream_));
  int rc = kOk;
  auto get = [&](auto& it) {
    if (rc == kOk) rc = download_as(it.V[p], v, nt);
    if (rc == kOk) rc = download_as(it.V[p ^ 1], v_new, nt);
    if (rc == kOk) rc = download_as(it.Y[p], y, m);
    if (rc == kOk) rc = download_as(it.Y[p ^ 1], y_new, m);
    if (rc == kOk) rc = download_as(it.Verg, v_erg, nt);
    if (rc == kOk) rc = download_as(it.Yerg, y_erg, m);
  };
  if (seam_fp32_) {
    get(it32_);
  } else {
    get(it64_);
  }
  return rc;
}

namespace {

template <typename T>
int time_steps(Ctl* c, const OpView<T>& Ks, const OpView<T>& K, const OpView<T>& Kt,
               const IterView<T>& it, const EvalView& ev, const RedView& red, int gsk, int gst,
               int gk, int gt, bool halpern, int reps, cudaStream_t s, double* ms) {
  cudaEvent_t e[4];
  for (auto& x : e) {
    if (cudaEventCreate(&x) != cudaSuccess) return kErrCuda;
  }
  // The step kernels the solve runs (classic or Halpern).
  auto dual = [&](int r) {
    if (halpern) {
      launch_halpern_dual(c, Ks, it, r, gsk, s);
    } else {
      launch_dual_step(c, Ks, it, r, gsk, s);
    }
  };
  auto primal = [&](int r) {
    if (halpern) {
      launch_halpern_primal(c, Kt, it, r, gst, s);
    } else {
      launch_primal_step(c, Kt, it, r, gst, s);
    }
  };
  for (int r = 0; r < 2; ++r) {
    dual(r);
    primal(r);
  }
  cudaEventRecord(e[0], s);
  for (int r = 0; r < reps; ++r) dual(r & 1);
  cudaEventRecord(e[1], s);
  for (int r = 0; r < reps; ++r) primal(r & 1);
  cudaEventRecord(e[2], s);
  for (int r = 0; r < reps; ++r) launch_eval(c, K, Kt, it, ev, red, gk, gt, 0, s, halpern);
  cudaEventRecord(e[3], s);
  const cudaError_t err = cudaEventSynchronize(e[3]);
  float a = 0, b = 0, d = 0;
  cudaEventElapsedTime(&a, e[0], e[1]);
  cudaEventElapsedTime(&b, e[1], e[2]);
  cudaEventElapsedTime(&d, e[2], e[3]);
  ms[0] = a / reps;
  ms[1] = b / reps;
  ms[2] = d / reps;
  for (auto& x : e) cudaEventDestroy(x);
  return err == cudaSuccess ? kOk : kErrCuda;
}

}  // namespace

int Engine::time_kernels(int reps, double* ms_dual, double* ms_primal, double* ms_eval) {
  std::string* err = nullptr;
  Ctl* c = fp32_ ? ctl32_ : ctl_;
  SG_TRY(cudaStreamSynchronize(stream_));
  Ctl h;
  SG_TRY(cudaMemcpy(&h, c, sizeof(Ctl), cudaMemcpyDeviceToHost));
  h.done = 0;
  h.t = 0;
  h.k = 0;
  h.max_iter = std::numeric_limits<long long>::max();
  SG_TRY(cudaMemcpy(c, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  double ms[3] = {0, 0, 0};
  int rc;
  if (fp32_) {
    IterView<float> it = iter_view(it32_);
    it.rhs = it32_.rhs;
    rc = time_steps(c, K_.step32(), K_.view32(), Kt_.view32(), it, inner_eval_view(), red_view(),
                    grid_step_k_, grid_step_t_, grid_k_, grid_t_, opt_.algorithm == 2, reps,
                    stream_, ms);
  } else {
    rc = time_steps(c, K_.step64(), K_.view64(), Kt_.view64(), iter_view(it64_), eval_view(), red_view(),
                    grid_step_k_, grid_step_t_, grid_k_, grid_t_, opt_.algorithm == 2, reps,
                    stream_, ms);
  }
  if (rc != kOk) return rc;
  *ms_dual = ms[0];
  *ms_primal = ms[1];
  *ms_eval = ms[2];
  h.done = 1;
  SG_TRY(cudaMemcpy(c, &h, sizeof(Ctl), cudaMemcpyHostToDevice));
  return kOk;
}

int Engine::spmv(int transpose, const double* x, double* y) {
  std::string* err = nullptr;
  const DevOp& op = transpose ? Kt_ : K_;
  double* dx = nullptr;
  double* dy = nullptr;
  SG_TRY(dalloc(&dx, static_cast<size_t>(op.cols)));
  SG_TRY(dalloc(&dy, static_cast<size_t>(op.rows)));
  SG_TRY(cudaMemcpy(dx, x, static_cast<size_t>(op.cols) * sizeof(double), cudaMemcpyHostToDevice));
  OpView<double> v = op.view64();
  v.val = op.val_orig;
  launch_spmv(v, dx, dy, std::max(1, std::min(op.ntiles, 65535)), stream_);
  SG_TRY(cudaGetLastError());
  SG_TRY(cudaStreamSynchronize(stream_));
  SG_TRY(cudaMemcpy(y, dy, static_cast<size_t>(op.rows) * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(dx);
  cudaFree(dy);
  return kOk;
}

}  // namespace sg

// mlp_engine.cpp -- host side of the GB300 MLP local-search engine.
#include "mlp_engine.h"

#include <algorithm>
#include <cctype>
#include <iterator>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "mlp_kernels.cuh"

namespace mlp {

namespace {
thread_local std::string g_last_error;

size_t al(size_t v) { return (v + 255) / 256 * 256; }
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return kOk;
  set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
  return e == cudaErrorMemoryAllocation ? kErrNoMem : kErrCuda;
}

#define MLP_CUDA(call, what)                        \
  do {                                              \
    int st_ = cuda_status((call), what);            \
    if (st_ != kOk) return st_;                     \
  } while (0)

// ---------------------------------------------------------------- Problem
Problem::~Problem() {
  if (async_alloc) {
    if (dD) cudaFreeAsync(dD, alloc_stream);
    if (dX) cudaFreeAsync(dX, alloc_stream);
    if (dY) cudaFreeAsync(dY, alloc_stream);
    return;
  }
  if (dD) cudaFree(dD);
  if (dX) cudaFree(dX);
  if (dY) cudaFree(dY);
}

static int check_n(int n, int cost_tour) {
  if (cost_tour != 1) {
    set_error("only costTour = 1 (closed tour with the depot repeated at the end) is supported; "
              "the reference's Or-opt kernels read past the tour for paths");
    return kErrUnsupported;
  }
  if (n < 5 || n + 1 > kMaxSize) {
    set_error("instance size out of range: need 5 <= n and n + 1 <= 16384 (14-bit move indices)");
    return kErrRange;
  }
  return kOk;
}

int problem_from_coords(int n, const int32_t* x, const int32_t* y, int cost_tour, int dist_round,
                        bool on_device, Problem** out) {
  if (!x || !y || !out) {
    set_error("null argument");
    return kErrArg;
  }
  int st = check_n(n, cost_tour);
  if (st != kOk) return st;
  std::unique_ptr<Problem> p(new Problem());
  p->n = n;
  p->size = n + cost_tour;
  p->cost_tour = cost_tour;
  p->dist_round = dist_round ? 1 : 0;
  MLP_CUDA(cudaGetDevice(&p->device), "cudaGetDevice");
  MLP_CUDA(cudaMalloc(&p->dX, sizeof(int32_t) * n), "cudaMalloc(coords)");
  MLP_CUDA(cudaMalloc(&p->dY, sizeof(int32_t) * n), "cudaMalloc(coords)");
  MLP_CUDA(cudaMalloc(&p->dD, sizeof(int32_t) * (size_t)n * n + 16), "cudaMalloc(D)");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  MLP_CUDA(cudaMemcpy(p->dX, x, sizeof(int32_t) * n, kind), "copy coords");
  MLP_CUDA(cudaMemcpy(p->dY, y, sizeof(int32_t) * n, kind), "copy coords");
  p->hx.resize(n);
  p->hy.resize(n);
  MLP_CUDA(cudaMemcpy(p->hx.data(), p->dX, sizeof(int32_t) * n, cudaMemcpyDeviceToHost), "copy coords");
  MLP_CUDA(cudaMemcpy(p->hy.data(), p->dY, sizeof(int32_t) * n, cudaMemcpyDeviceToHost), "copy coords");
  {
    const auto mmx = std::minmax_element(p->hx.begin(), p->hx.end());
    const auto mmy = std::minmax_element(p->hy.begin(), p->hy.end());
    if ((int64_t)*mmx.second - *mmx.first > 32767 || (int64_t)*mmy.second - *mmy.first > 32767) {
      set_error("coordinate spans must not exceed 32767 so that dx*dx + dy*dy fits int32");
      return kErrRange;
    }
  }
  int32_t* dmax = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(p->dD) + sizeof(int32_t) * (size_t)n * n);
  MLP_CUDA(cudaMemset(dmax, 0, sizeof(int32_t)), "memset");
  MLP_CUDA(launch_dist(p->dX, p->dY, n, p->dist_round, p->dD, dmax, 0), "dist kernel");
  MLP_CUDA(cudaMemcpy(&p->dmax, dmax, sizeof(int32_t), cudaMemcpyDeviceToHost), "dist kernel");
  if (p->dmax > kMaxDist) {
    set_error("a distance exceeds 65535 (the reference stores weights as ushort)");
    return kErrRange;
  }
  *out = p.release();
  return kOk;
}

int problem_from_coords_async(int n, const int32_t* x, const int32_t* y, int dist_round, cudaMemPool_t pool,
                              cudaStream_t stream, Problem** out) {
  if (!x || !y || !out) {
    set_error("null argument");
    return kErrArg;
  }
  int st = check_n(n, 1);
  if (st != kOk) return st;
  const auto mmx = std::minmax_element(x, x + n);
  const auto mmy = std::minmax_element(y, y + n);
  if ((int64_t)*mmx.second - *mmx.first > 32767 || (int64_t)*mmy.second - *mmy.first > 32767) {
    // spans <= 32767 also bound every distance by 46341 < 65535
    set_error("coordinate spans must not exceed 32767 so that dx*dx + dy*dy fits int32");
    return kErrRange;
  }
  std::unique_ptr<Problem> p(new Problem());
  p->n = n;
  p->size = n + 1;
  p->cost_tour = 1;
  p->dist_round = dist_round ? 1 : 0;
  p->alloc_stream = stream;
  p->async_alloc = true;
  p->dmax = 46341;
  MLP_CUDA(cudaGetDevice(&p->device), "cudaGetDevice");
  MLP_CUDA(cudaMallocFromPoolAsync(&p->dX, sizeof(int32_t) * n, pool, stream), "cudaMallocAsync(coords)");
  MLP_CUDA(cudaMallocFromPoolAsync(&p->dY, sizeof(int32_t) * n, pool, stream), "cudaMallocAsync(coords)");
  MLP_CUDA(cudaMallocFromPoolAsync(&p->dD, sizeof(int32_t) * (size_t)n * n + 16, pool, stream),
           "cudaMallocAsync(D)");
  // Pageable sources: the copies are staged before the calls return.
  MLP_CUDA(cudaMemcpyAsync(p->dX, x, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream), "copy coords");
  MLP_CUDA(cudaMemcpyAsync(p->dY, y, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream), "copy coords");
  int32_t* dmax = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(p->dD) + sizeof(int32_t) * (size_t)n * n);
  MLP_CUDA(cudaMemsetAsync(dmax, 0, sizeof(int32_t), stream), "memset");
  MLP_CUDA(launch_dist(p->dX, p->dY, n, p->dist_round, p->dD, dmax, stream), "dist kernel");
  *out = p.release();
  return kOk;
}

int problem_from_matrix(int n, const int32_t* D, int cost_tour, bool on_device, Problem** out) {
  if (!D || !out) {
    set_error("null argument");
    return kErrArg;
  }
  int st = check_n(n, cost_tour);
  if (st != kOk) return st;
  std::vector<int32_t> h;
  const int32_t* hd = D;
  if (on_device) {
    h.resize((size_t)n * n);
    MLP_CUDA(cudaMemcpy(h.data(), D, sizeof(int32_t) * (size_t)n * n, cudaMemcpyDeviceToHost), "copy D");
    hd = h.data();
  }
  int32_t mx = 0;
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) {
      const int32_t v = hd[(size_t)i * n + j];
      if (v < 0 || v > kMaxDist) {
        set_error("distances must lie in [0, 65535] (the reference stores weights as ushort)");
        return kErrRange;
      }
      if (v != hd[(size_t)j * n + i]) {
        set_error("the distance matrix must be symmetric (the move deltas assume d(a,b) = d(b,a))");
        return kErrArg;
      }
      mx = std::max(mx, v);
    }
  }
  std::unique_ptr<Problem> p(new Problem());
  p->n = n;
  p->size = n + cost_tour;
  p->cost_tour = cost_tour;
  p->dmax = mx;
  MLP_CUDA(cudaGetDevice(&p->device), "cudaGetDevice");
  MLP_CUDA(cudaMalloc(&p->dD, sizeof(int32_t) * (size_t)n * n + 16), "cudaMalloc(D)");
  MLP_CUDA(cudaMemcpy(p->dD, hd, sizeof(int32_t) * (size_t)n * n, cudaMemcpyHostToDevice), "copy D");
  *out = p.release();
  return kOk;
}

// TSPLIB header + NODE_COORD_SECTION reader; coordinates are read as float and
// rounded with nint (TSPLibInstance::inear, source/tsplib.cpp:237-240), as
// MLProblem::load does (source/mlproblem.cpp:116-117).
int read_tsplib_euc2d(const char* path, std::vector<int32_t>& x, std::vector<int32_t>& y,
                      std::string& name) {
  std::ifstream f(path);
  if (!f.is_open()) {
    set_error(std::string("cannot open instance file: ") + (path ? path : "(null)"));
    return kErrIo;
  }
  auto trim = [](const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
  };
  std::string line;
  int dim = -1;
  std::string ewt;
  bool coords = false;
  while (std::getline(f, line)) {
    size_t c = line.find(':');
    std::string key = trim(c == std::string::npos ? line : line.substr(0, c));
    std::string val = c == std::string::npos ? std::string() : trim(line.substr(c + 1));
    if (key == "NAME") name = val;
    else if (key == "DIMENSION") dim = std::atoi(val.c_str());
    else if (key == "EDGE_WEIGHT_TYPE") ewt = val;
    else if (key == "NODE_COORD_SECTION") {
      coords = true;
      break;
    }
  }
  if (ewt != "EUC_2D") {
    set_error("invalid instance: only EUC_2D coordinates are supported (source/mlproblem.cpp:94-95)");
    return kErrFormat;
  }
  if (!coords || dim <= 0) {
    set_error("invalid instance: missing DIMENSION or NODE_COORD_SECTION");
    return kErrFormat;
  }
  x.resize(dim);
  y.resize(dim);
  for (int i = 0; i < dim; i++) {
    int id;
    float fx, fy;
    if (!(f >> id >> fx >> fy)) {
      set_error("invalid instance: truncated NODE_COORD_SECTION");
      return kErrFormat;
    }
    x[i] = fx >= 0 ? (int)(fx + 0.5F) : (int)(fx - 0.5F);
    y[i] = fy >= 0 ? (int)(fy + 0.5F) : (int)(fy - 0.5F);
  }
  return kOk;
}

int problem_from_tsplib(const char* path, int cost_tour, int dist_round, Problem** out) {
  std::vector<int32_t> x, y;
  std::string name;
  int st = read_tsplib_euc2d(path, x, y, name);
  if (st != kOk) return st;
  st = problem_from_coords((int)x.size(), x.data(), y.data(), cost_tour, dist_round, false, out);
  if (st == kOk) (*out)->name = name;
  return st;
}

// ---------------------------------------------------------------- Job
size_t job_bytes(int size, bool wide, int moves_cap) {
  const size_t pad = size + 8, tb = total_blocks(size), cw = wide ? 8 : 4;
  size_t b = 0;
  b += al(4 * (size_t)size) * 2;        // tour, tour_alt
  b += al(4 * pad);                     // w
  b += al(cw * pad) * 2;                // W, Q
  b += al(4 * 3 * pad);                 // A
  b += al(8 * tb);                      // keys
  b += al(16 * tb);                     // kept
  b += al(4 * 8);                       // kept_count
  b += al(8 * kStatWords);              // stats
  b += al(4 * (size_t)moves_cap) + al(8 * (size_t)moves_cap);
  if (!wide) b += al(4 * kTermWords * (size_t)size) * 2;  // RT, CT
  if (merge_needs_ws(size)) b += al(merge_ws_bytes(size));
  return b;
}

Job::~Job() {
  if (total) cudaFree(total);
  if (!arena) return;
  if (async_alloc) cudaFreeAsync(arena, alloc_stream);
  else cudaFree(arena);
}

size_t job_total_bytes(int size, bool wide) {
  const size_t kept = (size_t)region_off(kNumNb, size);
  return al(4 * kNumNb) * 2 + al(8 * kept) + al(4 * kept) +
         al((size_t)total_list_off(kNumNb, size) * (wide ? 16 : 8));
}

int job_enable_total(Job* j) {
  if (j->total) return kOk;
  const size_t bytes = job_total_bytes(j->size, j->wide);
  MLP_CUDA(cudaMalloc(&j->total, bytes), "cudaMalloc(TOTAL lists)");
  const size_t kept = (size_t)region_off(kNumNb, j->size);
  char* c = static_cast<char*>(j->total);
  JobDev& d = j->dev;
  d.tcount = (int32_t*)c;  c += al(4 * kNumNb);
  d.tkcount = (int32_t*)c;  c += al(4 * kNumNb);
  d.tkcost = (int64_t*)c;  c += al(8 * kept);
  d.tkij = (uint32_t*)c;  c += al(4 * kept);
  d.tlist = c;
  j->total_bytes = bytes;
  MLP_CUDA(cudaMemset(j->total, 0, al(4 * kNumNb) * 2), "memset(TOTAL counters)");
  return kOk;
}

static void job_layout(Job* j, Problem* p, bool wide, int moves_cap);

int job_create(Problem* p, bool wide, int moves_cap, Job** out) {
  std::unique_ptr<Job> j(new Job());
  j->arena_bytes = job_bytes(p->size, wide, moves_cap);
  MLP_CUDA(cudaMalloc(&j->arena, j->arena_bytes), "cudaMalloc(job)");
  MLP_CUDA(cudaMemset(j->arena, 0, j->arena_bytes), "memset(job)");
  job_layout(j.get(), p, wide, moves_cap);
  *out = j.release();
  return kOk;
}

int job_create_async(Problem* p, bool wide, cudaMemPool_t pool, cudaStream_t stream, Job** out) {
  std::unique_ptr<Job> j(new Job());
  j->arena_bytes = job_bytes(p->size, wide, 0);
  j->alloc_stream = stream;
  j->async_alloc = true;
  MLP_CUDA(cudaMallocFromPoolAsync(&j->arena, j->arena_bytes, pool, stream), "cudaMallocAsync(job)");
  MLP_CUDA(cudaMemsetAsync(j->arena, 0, j->arena_bytes, stream), "memset(job)");
  job_layout(j.get(), p, wide, 0);
  *out = j.release();
  return kOk;
}

static void job_layout(Job* j, Problem* p, bool wide, int moves_cap) {
  j->prob = p;
  j->wide = wide;
  j->size = p->size;
  j->moves_cap = moves_cap;
  const int size = p->size;
  const size_t pad = size + 8, tb = total_blocks(size), cw = wide ? 8 : 4;
  char* c = static_cast<char*>(j->arena);
  JobDev& d = j->dev;
  d.D = p->dD;
  d.tour = (int32_t*)c;  c += al(4 * (size_t)size);
  d.tour_alt = (int32_t*)c;  c += al(4 * (size_t)size);
  d.w = (int32_t*)c;  c += al(4 * pad);
  d.W = c;  c += al(cw * pad);
  d.Q = c;  c += al(cw * pad);
  d.A = (int32_t*)c;  c += al(4 * 3 * pad);
  d.keys = (uint64_t*)c;  c += al(8 * tb);
  d.kept = (uint64_t*)c;  c += al(16 * tb);
  d.kept_count = (int32_t*)c;  c += al(4 * 8);
  d.stats = (int64_t*)c;  c += al(8 * kStatWords);
  d.moves_out = moves_cap > 0 ? (uint32_t*)c : nullptr;  c += al(4 * (size_t)moves_cap);
  d.moves_cost = moves_cap > 0 ? (int64_t*)c : nullptr;  c += al(8 * (size_t)moves_cap);
  d.RT = d.CT = nullptr;
  if (!wide) {
    d.RT = j->rt_mem = (int32_t*)c;  c += al(4 * kTermWords * (size_t)size);
    d.CT = j->ct_mem = (int32_t*)c;  c += al(4 * kTermWords * (size_t)size);
  }
  d.ws = nullptr;
  if (merge_needs_ws(size)) {
    d.ws = (uint8_t*)c;
    c += al(merge_ws_bytes(size));
  }
  d.moves_cap = moves_cap;
  d.n = p->n;
  d.size = size;
  d.nb_mask = 0x1f;
  d.flags = wide ? kFlagWide : 0;
}

void job_tiles(int size, int shape, std::vector<SweepTile>* out) {
  const TileShape ts = kTileShapes[shape];
  out->clear();
  for (int rb = 0; rb < sweep_row_blocks(size, ts.tr); rb++) {
    const int r0 = 1 + rb * ts.tr;
    for (int c = 0; c < sweep_row_tiles(size, r0, ts.tl); c++) out->push_back(SweepTile{0, r0, 1 + c * ts.tl, 0});
  }
}

// Tile-shape table chosen by the autotuner (mlpgpu/autotune.py): rows of
// (largest tour size, shape for one job, shape for many jobs), ascending.
namespace {
std::mutex g_tune_mu;
std::vector<std::array<int32_t, 3>> g_tune;
}  // namespace

int tuning_set(const int32_t* max_size, const int32_t* one, const int32_t* many, int count) {
  if (count < 0 || count > 64 || (count > 0 && (!max_size || !one || !many))) {
    set_error("tuning table: count must lie in [0, 64] with three arrays of that length");
    return kErrArg;
  }
  std::vector<std::array<int32_t, 3>> t;
  for (int q = 0; q < count; q++) {
    if (max_size[q] < 1 || one[q] < 0 || one[q] >= kNumTileShapes || many[q] < 0 || many[q] >= kNumTileShapes) {
      set_error("tuning table: sizes must be positive and shapes valid tile-shape indices");
      return kErrArg;
    }
    if (q > 0 && max_size[q] <= max_size[q - 1]) {
      set_error("tuning table: sizes must be strictly increasing");
      return kErrArg;
    }
    t.push_back({max_size[q], one[q], many[q]});
  }
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.swap(t);
  return kOk;
}

int tuning_get(int32_t* max_size, int32_t* one, int32_t* many, int cap, int* count) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (count) *count = (int)g_tune.size();
  for (int q = 0; q < (int)g_tune.size() && q < cap; q++) {
    if (max_size) max_size[q] = g_tune[q][0];
    if (one) one[q] = g_tune[q][1];
    if (many) many[q] = g_tune[q][2];
  }
  return kOk;
}

int tuning_load(const char* path) {
  std::ifstream f(path ? path : "");
  if (!f.is_open()) {
    set_error(std::string("cannot open tuning table: ") + (path ? path : "(null)"));
    return kErrIo;
  }
  // The integers of the "table" array, three per row ([size, one, many]).
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  const size_t k = text.find("\"table\"");
  if (k == std::string::npos) {
    set_error("tuning table: no \"table\" key");
    return kErrFormat;
  }
  const size_t open = text.find('[', k);
  if (open == std::string::npos) {
    set_error("tuning table: \"table\" must be a list of [size, shape_one, shape_many] rows");
    return kErrFormat;
  }
  std::vector<int32_t> v;
  int depth = 0;
  size_t q = open;
  for (; q < text.size(); q++) {
    const char ch = text[q];
    if (ch == '[') depth++;
    else if (ch == ']' && --depth == 0) break;
    else if (std::isdigit((unsigned char)ch)) {
      size_t e = q;
      while (e < text.size() && std::isdigit((unsigned char)text[e])) e++;
      v.push_back((int32_t)std::atol(text.substr(q, e - q).c_str()));
      q = e - 1;
    }
  }
  if (depth != 0) {
    set_error("tuning table: unterminated \"table\" list");
    return kErrFormat;
  }
  if (v.empty() || v.size() % 3 != 0) {
    set_error("tuning table: rows must hold three integers");
    return kErrFormat;
  }
  std::vector<int32_t> a, b, c;
  for (size_t q = 0; q < v.size(); q += 3) {
    a.push_back(v[q]);
    b.push_back(v[q + 1]);
    c.push_back(v[q + 2]);
  }
  return tuning_set(a.data(), b.data(), c.data(), (int)a.size());
}

int default_shape(int size, int njobs) {
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (const auto& row : g_tune)
      if (size <= row[0]) return njobs >= kManyJobs ? row[2] : row[1];
  }
  // Built-in rule, measured on GB300: one n=1000 job is latency-bound and
  // prefers many small tiles; a set of many jobs is throughput-bound and
  // prefers 64 x 8.
  if (size > 2000) return 7;          // 128 diagonals x 16 rows
  if (njobs >= kManyJobs) return 4;   // 64 x 8
  if (size <= 400) return 0;          // 32 x 4
  return 3;                           // 64 x 4
}

// ---------------------------------------------------------------- constructor
int check_alpha(float alpha) {
  if (!(alpha >= 0.0f && alpha <= 1.0f)) {
    set_error("alpha must lie in [0, 1]");
    return kErrArg;
  }
  return kOk;
}

int build_random_tours(const std::vector<GraspTask>& tasks, cudaStream_t stream) {
  if (tasks.empty()) return kOk;
  struct Buffers {  // stream-ordered: no device-wide synchronisation
    cudaStream_t st;
    GraspTask* tasks = nullptr;
    int* err = nullptr;
    uint32_t* scratch = nullptr;
    ~Buffers() {
      if (tasks) cudaFreeAsync(tasks, st);
      if (err) cudaFreeAsync(err, st);
      if (scratch) cudaFreeAsync(scratch, st);
    }
  } b{stream};
  // Canonical-tie tasks first, then the reference-tie ones (one launch each);
  // the latter above kGraspRefSmemN nodes get 2n words of scratch.
  std::vector<GraspTask> order;
  int64_t words = 0;
  for (int pass = 0; pass < 2; pass++)
    for (GraspTask t : tasks) {
      if (t.n < 1 || t.n > kMaxSize - 1 || !t.D || !t.tour || t.ties < 0 || t.ties > 1) {
        set_error("constructor task out of range");
        return kErrArg;
      }
      if (t.ties != pass) continue;
      t.scratch = 0;
      if (t.ties && t.n > kGraspRefSmemN) {
        t.scratch = words;
        words += 2 * (int64_t)t.n;
      }
      order.push_back(t);
    }
  int ncanon = 0;
  while (ncanon < (int)order.size() && order[ncanon].ties == 0) ncanon++;
  MLP_CUDA(cudaMallocAsync(&b.tasks, sizeof(GraspTask) * order.size(), stream), "cudaMallocAsync(constructor tasks)");
  MLP_CUDA(cudaMallocAsync(&b.err, sizeof(int), stream), "cudaMallocAsync(constructor flag)");
  if (words > 0)
    MLP_CUDA(cudaMallocAsync(&b.scratch, sizeof(uint32_t) * (size_t)words, stream),
             "cudaMallocAsync(constructor scratch)");
  MLP_CUDA(cudaMemcpyAsync(b.tasks, order.data(), sizeof(GraspTask) * order.size(), cudaMemcpyHostToDevice,
                           stream),
           "copy constructor tasks");
  MLP_CUDA(cudaMemsetAsync(b.err, 0, sizeof(int), stream), "memset(constructor flag)");
  MLP_CUDA(launch_grasp(b.tasks, ncanon, 0, nullptr, b.err, stream), "constructor kernel");
  MLP_CUDA(launch_grasp(b.tasks + ncanon, (int)order.size() - ncanon, 1, b.scratch, b.err, stream),
           "constructor kernel");
  int herr = 0;
  MLP_CUDA(cudaMemcpyAsync(&herr, b.err, sizeof(int), cudaMemcpyDeviceToHost, stream), "read constructor flag");
  MLP_CUDA(cudaStreamSynchronize(stream), "constructor");
  if (herr) {
    set_error("device constructor failed an internal check");
    return kErrState;
  }
  return kOk;
}

// ---------------------------------------------------------------- JobSet
JobSet::JobSet(std::vector<Job*> jobs, bool wide, cudaStream_t stream)
    : all_jobs_(jobs), jobs_(std::move(jobs)), wide_(wide), stream_(stream) {}

JobSet::~JobSet() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
  if (djobs_) cudaFree(djobs_);
  if (dtiles_) cudaFree(dtiles_);
  if (hstats_) cudaFreeHost(hstats_);
  if (hstats2_) cudaFreeHost(hstats2_);
  for (int b = 0; b < 2; b++) {
    if (stats_ev_[b]) cudaEventDestroy(stats_ev_[b]);
    if (htiles_[b]) cudaFreeHost(htiles_[b]);
    if (hjobs_[b]) cudaFreeHost(hjobs_[b]);
  }
  if (dstats_) cudaFree(dstats_);
  for (void* p : extra_ws_) cudaFree(p);
}

int JobSet::init() {
  if (jobs_.empty()) {
    set_error("empty job set");
    return kErrArg;
  }
  max_size_ = 0;
  for (Job* j : jobs_) {
    if (j->wide != wide_) {
      set_error("all jobs of a set must share the cost width");
      return kErrArg;
    }
    max_size_ = std::max(max_size_, j->size);
  }
  merge_smem_ = max_size_ <= merge_smem_max_size();
  solo_smem_ = max_size_ <= solo_smem_max_size();
  if (!merge_smem_ || !solo_smem_) {
    // The merge runs from global workspaces: give one to every job lacking it.
    for (Job* j : jobs_) {
      if (j->dev.ws != nullptr) continue;
      void* p = nullptr;
      MLP_CUDA(cudaMalloc(&p, merge_ws_bytes(j->size)), "cudaMalloc(merge workspace)");
      extra_ws_.push_back(p);
      j->dev.ws = static_cast<uint8_t*>(p);
    }
  }
  MLP_CUDA(configure_merge(merge_smem_ ? merge_smem_bytes(max_size_) : 0), "configure merge");
  MLP_CUDA(cudaMallocHost(&hstats_, sizeof(int64_t) * kStatWords * jobs_.size()), "cudaMallocHost");
  MLP_CUDA(cudaMallocHost(&hstats2_, sizeof(int64_t) * kStatWords * jobs_.size()), "cudaMallocHost");
  for (int b = 0; b < 2; b++) {
    MLP_CUDA(cudaEventCreateWithFlags(&stats_ev_[b], cudaEventDisableTiming), "event");
    MLP_CUDA(cudaMallocHost(&hjobs_[b], sizeof(JobDev) * jobs_.size()), "cudaMallocHost");
  }
  MLP_CUDA(cudaMalloc(&dstats_, sizeof(int64_t) * kStatWords * jobs_.size()), "cudaMalloc(stats)");
  MLP_CUDA(cudaMemset(dstats_, 0, sizeof(int64_t) * kStatWords * jobs_.size()), "memset(stats)");
  MLP_CUDA(cudaMalloc(&djobs_, sizeof(JobDev) * jobs_.size()), "cudaMalloc(jobs)");
  JobDev* h = hjobs_[0];
  for (size_t q = 0; q < jobs_.size(); q++) {
    jobs_[q]->dev.stats = dstats_ + q * kStatWords;
    jobs_[q]->dev.RT = local_terms() ? nullptr : jobs_[q]->rt_mem;
    jobs_[q]->dev.CT = local_terms() ? nullptr : jobs_[q]->ct_mem;
    h[q] = jobs_[q]->dev;
  }
  MLP_CUDA(cudaMemcpyAsync(djobs_, h, sizeof(JobDev) * jobs_.size(), cudaMemcpyHostToDevice, stream_),
           "copy jobs");
  MLP_CUDA(cudaStreamSynchronize(stream_), "copy jobs");
  if (shape_ < 0) shape_ = default_shape(max_size_, (int)jobs_.size());
  return build_tiles();
}

int JobSet::build_tiles(int buf, bool sync) {
  const TileShape ts = kTileShapes[shape_];
  size_t count = 0;
  for (size_t q = 0; q < jobs_.size(); q++) {
    const int sz = jobs_[q]->size;
    for (int rb = 0; rb < sweep_row_blocks(sz, ts.tr); rb++) count += (size_t)sweep_row_tiles(sz, 1 + rb * ts.tr, ts.tl);
  }
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
  loop_graph_ = nullptr;
  if (count > tiles_cap_ || dtiles_ == nullptr) {
    // Grow (the set's first build, or more jobs or smaller tiles than before).
    MLP_CUDA(cudaStreamSynchronize(stream_), "grow tiles");
    if (dtiles_) cudaFree(dtiles_);
    dtiles_ = nullptr;
    for (int b = 0; b < 2; b++) {
      if (htiles_[b]) cudaFreeHost(htiles_[b]);
      htiles_[b] = nullptr;
    }
    tiles_cap_ = 0;
    const size_t cap = std::max<size_t>(1, count);
    MLP_CUDA(cudaMalloc(&dtiles_, sizeof(SweepTile) * cap), "cudaMalloc(tiles)");
    for (int b = 0; b < 2; b++) MLP_CUDA(cudaMallocHost(&htiles_[b], sizeof(SweepTile) * cap), "cudaMallocHost(tiles)");
    tiles_cap_ = cap;
  }
  SweepTile* h = htiles_[buf];
  size_t k = 0;
  for (size_t q = 0; q < jobs_.size(); q++) {
    const int sz = jobs_[q]->size;
    for (int rb = 0; rb < sweep_row_blocks(sz, ts.tr); rb++) {
      const int r0 = 1 + rb * ts.tr;
      for (int c = 0; c < sweep_row_tiles(sz, r0, ts.tl); c++) h[k++] = SweepTile{(int32_t)q, r0, 1 + c * ts.tl, 0};
    }
  }
  ntiles_ = (int)count;
  if (count > 0)
    MLP_CUDA(cudaMemcpyAsync(dtiles_, h, sizeof(SweepTile) * count, cudaMemcpyHostToDevice, stream_), "copy tiles");
  if (sync) MLP_CUDA(cudaStreamSynchronize(stream_), "copy tiles");
  return kOk;
}

int JobSet::set_active(const std::vector<int>& idx, int buf, bool sync) {
  std::vector<Job*> next;
  for (int q : idx) {
    if (q < 0 || q >= (int)all_jobs_.size()) {
      set_error("active job index out of range");
      return kErrArg;
    }
    next.push_back(all_jobs_[q]);
  }
  if (next == jobs_) return kOk;
  jobs_ = next;
  if (jobs_.empty()) return kOk;
  JobDev* h = hjobs_[buf];
  for (size_t q = 0; q < jobs_.size(); q++) h[q] = jobs_[q]->dev;
  MLP_CUDA(cudaMemcpyAsync(djobs_, h, sizeof(JobDev) * jobs_.size(), cudaMemcpyHostToDevice, stream_),
           "copy jobs");
  return build_tiles(buf, sync);
}

int JobSet::ensure_all_active() {
  if (jobs_.size() == all_jobs_.size()) return kOk;
  std::vector<int> all(all_jobs_.size());
  for (size_t q = 0; q < all.size(); q++) all[q] = (int)q;
  return set_active(all);
}

int JobSet::set_stream(cudaStream_t s) {
  stream_ = s;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
  loop_graph_ = nullptr;
  return kOk;
}

int JobSet::set_shape(int shape) {
  if (shape < 0 || shape >= kNumTileShapes) {
    set_error("tile shape index out of range");
    return kErrArg;
  }
  if (total_) {  // the collecting sweep has one shape; this one applies afterwards
    shape_user_ = shape;
    return kOk;
  }
  shape_ = shape;
  return djobs_ ? build_tiles() : kOk;
}

int JobSet::set_unroll(int u) {
  if (u < 1 || u > 256) {
    set_error("unroll out of range [1, 256]");
    return kErrArg;
  }
  unroll_ = u;
  return kOk;
}

int JobSet::set_mask(int mask) {
  if (mask <= 0 || mask > 0x1f) {
    set_error("neighbourhood mask must be a nonzero subset of 0x1f");
    return kErrArg;
  }
  if (mask == mask_) return kOk;
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  const bool was_dvnd = dvnd_sweep();
  mask_ = mask;
  if (dvnd_sweep() != was_dvnd) drop_graphs();  // the captured sweep kernel changes
  for (size_t q = 0; q < jobs_.size(); q++) {
    jobs_[q]->dev.nb_mask = mask;
    MLP_CUDA(cudaMemcpyAsync(&djobs_[q].nb_mask, &jobs_[q]->dev.nb_mask, sizeof(int32_t),
                             cudaMemcpyHostToDevice, stream_),
             "set mask");
  }
  MLP_CUDA(cudaStreamSynchronize(stream_), "set mask");
  return kOk;
}

int JobSet::set_record_moves(bool on) {
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  for (size_t q = 0; q < jobs_.size(); q++) {
    int32_t f = jobs_[q]->dev.flags;
    f = on ? (f | kFlagRecordMoves) : (f & ~kFlagRecordMoves);
    if (f == jobs_[q]->dev.flags) continue;
    jobs_[q]->dev.flags = f;
    MLP_CUDA(cudaMemcpyAsync(&djobs_[q].flags, &jobs_[q]->dev.flags, sizeof(int32_t), cudaMemcpyHostToDevice,
                             stream_),
             "set flags");
  }
  MLP_CUDA(cudaStreamSynchronize(stream_), "set flags");
  return kOk;
}

int JobSet::prepare(bool reset_stats) {
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  MLP_CUDA(launch_prepare(djobs_, (int)jobs_.size(), wide_, reset_stats, stream_), "prepare kernel");
  return kOk;
}

bool JobSet::solo_merge() const {
  return merge_mode_ == kMergeSolo || (merge_mode_ == kMergeAuto && (int)jobs_.size() >= kSoloMinJobs);
}

int JobSet::set_total(bool on) {
  if (on == total_) return kOk;
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  if (on) {
    for (Job* j : all_jobs_) {
      int st = job_enable_total(j);
      if (st != kOk) return st;
    }
    std::vector<JobDev> h(jobs_.size());
    for (size_t q = 0; q < jobs_.size(); q++) h[q] = jobs_[q]->dev;
    MLP_CUDA(cudaMemcpyAsync(djobs_, h.data(), sizeof(JobDev) * h.size(), cudaMemcpyHostToDevice, stream_),
             "copy jobs");
    MLP_CUDA(cudaStreamSynchronize(stream_), "copy jobs");
    shape_user_ = shape_;
    shape_ = total_shape(max_size_);
  } else {
    shape_ = shape_user_;
  }
  total_ = on;
  return build_tiles();  // also drops the captured graphs
}

int JobSet::launch_iteration() {
  if (total_) {
    const int nj = (int)jobs_.size();
    MLP_CUDA(launch_sweep_collect(dtiles_, ntiles_, djobs_, wide_, shape_, stream_), "sweep kernel");
    MLP_CUDA(launch_total_select(djobs_, nj, wide_, stream_), "TOTAL greedy kernel");
    MLP_CUDA(launch_total_finish(djobs_, nj, wide_, solo_smem_, max_size_, stream_), "merge kernel");
    return kOk;
  }
  if (dvnd_sweep())
    MLP_CUDA(launch_sweep_dvnd(dtiles_, ntiles_, djobs_, shape_, local_terms(), stream_), "sweep kernel");
  else
    MLP_CUDA(launch_sweep(dtiles_, ntiles_, djobs_, wide_, shape_, true, stream_), "sweep kernel");
  if (solo_merge())
    MLP_CUDA(launch_merge_solo(djobs_, (int)jobs_.size(), wide_, solo_smem_, max_size_, stream_), "merge kernel");
  else
    MLP_CUDA(launch_merge(djobs_, (int)jobs_.size(), wide_, merge_smem_, max_size_, stream_), "merge kernel");
  return kOk;
}

void JobSet::drop_graphs() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
  loop_graph_ = nullptr;
}

int JobSet::set_sweep_kernel(int variant) {
  if (variant < 0 || variant > 1) {
    set_error("sweep kernel must be 0 (general) or 1 (term tables)");
    return kErrArg;
  }
  if (variant == sweep_variant_) return kOk;
  sweep_variant_ = variant;
  drop_graphs();
  return kOk;
}

int JobSet::set_merge_mode(int mode) {
  if (mode < kMergeAuto || mode > kMergeSolo) {
    set_error("merge mode must be 0 (auto), 1 (cluster) or 2 (one CTA per job)");
    return kErrArg;
  }
  if (mode == merge_mode_) return kOk;
  merge_mode_ = mode;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
  loop_graph_ = nullptr;
  return kOk;
}

int JobSet::sweep_only() {
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  MLP_CUDA(launch_stats_begin(djobs_, (int)jobs_.size(), 1, stream_), "stats kernel");
  MLP_CUDA(launch_sweep(dtiles_, ntiles_, djobs_, wide_, shape_, false, stream_), "sweep kernel");
  return kOk;
}

int JobSet::sweep_kernel() {
  if (dvnd_sweep())
    MLP_CUDA(launch_sweep_dvnd(dtiles_, ntiles_, djobs_, shape_, local_terms(), stream_), "sweep kernel");
  else
    MLP_CUDA(launch_sweep(dtiles_, ntiles_, djobs_, wide_, shape_, true, stream_), "sweep kernel");
  return kOk;
}

int JobSet::graph_for(int iters, cudaGraphExec_t* out) {
  auto it = graphs_.find(iters);
  if (it != graphs_.end()) {
    *out = it->second;
    return kOk;
  }
  cudaGraph_t g;
  MLP_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
  for (int q = 0; q < iters; q++) {
    int st = launch_iteration();
    if (st != kOk) {
      cudaStreamEndCapture(stream_, &g);
      return st;
    }
  }
  MLP_CUDA(cudaStreamEndCapture(stream_, &g), "end capture");
  cudaGraphExec_t ge;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  MLP_CUDA(e, "graph instantiate");
  graphs_[iters] = ge;
  *out = ge;
  return kOk;
}

int JobSet::enqueue_iterations(int iters) {
  if (stream_ == 0) {
    for (int q = 0; q < iters; q++) {
      int st = launch_iteration();
      if (st != kOk) return st;
    }
    return kOk;
  }
  while (iters > 0) {
    const int u = std::min(iters, unroll_);
    cudaGraphExec_t ge;
    int st = graph_for(u, &ge);
    if (st != kOk) return st;
    MLP_CUDA(cudaGraphLaunch(ge, stream_), "graph launch");
    iters -= u;
  }
  return kOk;
}

// Iterations per pass of the device-side loop's body: the while node's
// condition kernel runs once per pass, and a search that converges within a
// pass leaves the rest of it as kernels that return at once.
constexpr int kDeviceLoopBody = 16;

int JobSet::enqueue_device_loop(int max_iters) {
  if (max_iters <= 0) {
    set_error("max_iters must be positive");
    return kErrArg;
  }
  if (stream_ == 0) {
    set_error("the device-side loop needs a non-default stream");
    return kErrState;
  }
  const int unroll = kDeviceLoopBody;
  if (!loop_graph_ || loop_unroll_ != unroll) {
    if (loop_graph_) cudaGraphExecDestroy(loop_graph_);
    loop_graph_ = nullptr;
    cudaGraph_t g;
    MLP_CUDA(cudaGraphCreate(&g, 0), "graph create");
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_status(e, "conditional handle");
    }
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_status(e, "conditional node");
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(stream_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_status(e, "capture body");
    }
    int st = kOk;
    for (int q = 0; q < unroll && st == kOk; q++) st = launch_iteration();
    if (st == kOk) st = cuda_status(launch_loop_condition(djobs_, (int)jobs_.size(), h, stream_), "condition kernel");
    cudaGraph_t captured;
    cudaError_t e2 = cudaStreamEndCapture(stream_, &captured);
    if (st != kOk) {
      cudaGraphDestroy(g);
      return st;
    }
    if (e2 != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_status(e2, "end capture");
    }
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    MLP_CUDA(e, "graph instantiate");
    loop_graph_ = ge;
    loop_unroll_ = unroll;
  }
  MLP_CUDA(launch_stats_begin(djobs_, (int)jobs_.size(), max_iters, stream_), "stats kernel");
  MLP_CUDA(cudaGraphLaunch(loop_graph_, stream_), "graph launch");
  return kOk;
}

int JobSet::run(int max_iters, bool sync) {
  if (max_iters <= 0) {
    set_error("max_iters must be positive");
    return kErrArg;
  }
  {
    int st = ensure_all_active();
    if (st != kOk) return st;
  }
  if (device_loop_ && stream_ != 0 && all_jobs_.size() == 1) {
    int st = enqueue_device_loop(max_iters);
    if (st != kOk || !sync) return st;
    std::vector<std::array<int64_t, kStatWords>> s;
    return read_stats(&s);
  }
  MLP_CUDA(launch_stats_begin(djobs_, (int)jobs_.size(), max_iters, stream_), "stats kernel");
  // Host-checked loop.  A single job replays CUDA graphs of `unroll`
  // iterations; a batch launches directly and, after every check, drops the
  // jobs that converged from the launches (grids shrink as the batch drains).
  const bool graphs = all_jobs_.size() == 1 && stream_ != 0;
  std::vector<int> active(all_jobs_.size());
  for (size_t q = 0; q < active.size(); q++) active[q] = (int)q;
  int done = 0;
  int st = kOk;
  if (!graphs && sync) {
    // A batch checks one chunk late: chunk k + 1 is enqueued before the host
    // waits for chunk k's statistics, so the device never waits for the
    // host.  Jobs that converge meanwhile stay in one more chunk, whose
    // kernels they leave at once; the new job and tile arrays go into the
    // stream behind the chunk in flight, staged in pinned buffer b, which is
    // staged into again only after the next check's wait (two chunks later).
    int64_t* hst[2] = {hstats_, hstats2_};
    const size_t sbytes = sizeof(int64_t) * kStatWords * all_jobs_.size();
    int pend = -1, b = 0;
    while (done < max_iters) {
      const int u = std::min(unroll_, max_iters - done);
      for (int q = 0; q < u && st == kOk; q++) st = launch_iteration();
      if (st != kOk) break;
      done += u;
      st = cuda_status(cudaMemcpyAsync(hst[b], dstats_, sbytes, cudaMemcpyDeviceToHost, stream_), "read stats");
      if (st == kOk) st = cuda_status(cudaEventRecord(stats_ev_[b], stream_), "read stats");
      if (st != kOk) break;
      if (pend >= 0) {
        st = cuda_status(cudaEventSynchronize(stats_ev_[pend]), "read stats");
        if (st == kOk) st = check_stats(hst[pend]);
        if (st != kOk) break;
        std::vector<int> next;
        for (int q : active) {
          const int64_t* sq = hst[pend] + (size_t)q * kStatWords;
          if (!sq[kStatConverged] && sq[kStatSweeps] < max_iters) next.push_back(q);
        }
        if (next.empty()) break;
        if (next.size() < active.size()) {
          st = set_active(next, b, false);
          if (st != kOk) break;
          active.swap(next);
        }
      }
      pend = b;
      b ^= 1;
    }
    const int st1 = cuda_status(cudaStreamSynchronize(stream_), "batch loop");
    if (st == kOk) st = st1;
    const int st2 = ensure_all_active();
    return st != kOk ? st : st2;
  }
  while (done < max_iters) {
    const int u = std::min(unroll_, max_iters - done);
    if (graphs) {
      st = enqueue_iterations(u);
    } else {
      for (int q = 0; q < u && st == kOk; q++) st = launch_iteration();
    }
    if (st != kOk) break;
    done += u;
    if (!sync && done < max_iters) continue;
    std::vector<std::array<int64_t, kStatWords>> s;
    st = read_stats(&s);
    if (st != kOk) break;
    std::vector<int> next;
    for (int q : active)
      if (!s[q][kStatConverged] && s[q][kStatSweeps] < max_iters) next.push_back(q);
    if (next.empty()) break;
    if (!graphs && next.size() < active.size()) {
      st = set_active(next);
      if (st != kOk) break;
      active.swap(next);
    }
  }
  const int st2 = ensure_all_active();
  return st != kOk ? st : st2;
}

int JobSet::read_stats(std::vector<std::array<int64_t, kStatWords>>* out) {
  MLP_CUDA(cudaMemcpyAsync(hstats_, dstats_, sizeof(int64_t) * kStatWords * all_jobs_.size(),
                           cudaMemcpyDeviceToHost, stream_),
           "read stats");
  MLP_CUDA(cudaStreamSynchronize(stream_), "read stats");
  out->resize(all_jobs_.size());
  for (size_t q = 0; q < all_jobs_.size(); q++)
    std::memcpy((*out)[q].data(), hstats_ + q * kStatWords, sizeof(int64_t) * kStatWords);
  return check_stats(hstats_);
}

int JobSet::check_stats(const int64_t* hst) {
  int64_t err = 0;
  for (size_t q = 0; q < all_jobs_.size(); q++) err |= hst[q * kStatWords + kStatError];
  if (err) {
    static const char* what[] = {"", "", "merge stage-2 hand-off timed out (no longer produced)", "kept-move region overflow",
                                 "TOTAL list overflow", "TOTAL selection invariant broken"};
    set_error(std::string("device reported an internal error (code ") + std::to_string(err) + ": " +
              (err >= 2 && err <= 5 ? what[err] : "unknown") + ")");
    return kErrState;
  }
  return kOk;
}

int64_t JobSet::evals_per_sweep(int job, int mask) const {
  const int sz = all_jobs_[job]->size;
  int64_t e = 0;
  for (int nb = 0; nb < kNumNb; nb++)
    if ((mask >> nb) & 1) e += (int64_t)nb_blocks(nb, sz) * nb_threads(nb, sz);
  return e;
}

}  // namespace mlp

// pc_mol.cu — C ABI of the GB300-native MOL right-hand side (include/pelec_mol.h).
//
// Host side: validation of the operator configuration and of the box
// descriptors, the device species tables, the per-level launch layout (box
// table, cell-chunk list of pass 1, tile list of pass 2) cached across calls
// with the same BoxArray, the scratch that holds the per-cell records, and
// the diagnostic counters.  Device side: pc_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "pc_adjoint.cuh"
#include "pc_kernels.cuh"
#include "pc_level.cuh"
#include "pc_mixed.cuh"
#include "pc_rcp.h"
#include "pelec_mol.h"

namespace pcg {
int launch_mixed(int nspec, int tile, bool persistent, bool strict, const DevBox* boxes, const int2* items,
                 int nitems, const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                 double p_ref, unsigned long long* counters, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1,
                 cudaEvent_t e2, const FluxBox* fx);
cudaError_t launch_flux_fp64_tile(int tile, bool persistent, int nspec, const DevBox* boxes, const int4* tiles,
                                  int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                                  unsigned long long* counters, cudaStream_t s, const FluxBox* fx);
cudaError_t launch_vjp_passes(int nspec, const DevBox* boxes, const AdjBox* adj, const int2* items, int nitems,
                              const int4* fitems, int nfitems, double* recbar, long long nrecbar,
                              const long long* recbar_off, const MechSet& ms, const DevFlags& f, const Geo& g,
                              unsigned long long* counters, cudaStream_t s);
cudaError_t launch_jvp_passes(int nspec, const DevBox* boxes, const TanBox* tans, const int2* items, int nitems,
                              const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                              unsigned long long* counters, cudaStream_t s);
}  // namespace pcg

namespace {

using namespace pcg;

struct Layout {
  std::vector<DevBox> boxes;
  std::vector<int2> items;
  std::vector<int4> tiles;
  std::vector<int> item_start, tile_start;  // per box, with a final sentinel
  size_t scratch_doubles = 0;
};

}  // namespace

struct pc_mol_handle {
  pc_mol_config cfg{};
  int device = 0;
  int variant = 0;  // the species count: 1 (GammaLaw/Constant), 9 or 21 (IdealMix/Simple)
  MechSet mech{};
  DevFlags flags{};
  int nrec = 0;
  unsigned long long* d_counters = nullptr;
  // layout cache
  std::vector<pc_box_desc> last_boxes;
  double last_dx[3] = {0, 0, 0};
  int lay_tile = -1;  // tile shape the cached layout was built for
  Layout lay;
  // flux-pass launch configuration (tile shape + kNumTiles if persistent):
  // forced by pc_mol_set_tile (>= 0), else looked up in the autotune cache by
  // the BoxArray's box-size multiset, else 0
  int tile_forced = -1;
  int tile = 0;
  std::map<std::vector<int>, int> tune_cache;
  int smem_optin = 0;  // shared memory a CTA may opt into on the device (bytes)
  // Device box tables of the current layout, one per set of array pointers
  // (callers alternate a few state/RHS buffers; a pointer change must not
  // cost a layout rebuild).  d_boxes is the table of the last call.
  struct BoxTable {
    std::vector<pc_box_desc> key;
    std::vector<DevBox> host;
    DevBox* dev = nullptr;
    size_t cap = 0;
    unsigned long long stamp = 0;
  };
  BoxTable tables[4];
  unsigned long long table_clock = 0;
  DevBox* d_boxes = nullptr;
  int2* d_items = nullptr;
  size_t cap_items = 0;
  int4* d_tiles = nullptr;
  size_t cap_tiles = 0;
  double* scratch = nullptr;
  size_t scratch_cap = 0;  // doubles
  cudaStream_t last_stream = nullptr;
  int last_error = PC_OK;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // pass timing (cfg.time_passes)
  bool timed = false;
  // level operations: uploads cached by content (see upload())
  struct Upload {
    std::vector<unsigned char> host;
    void* dev = nullptr;
    size_t cap = 0;
  };
  Upload up[12];
  unsigned long long* d_dt = nullptr;  // 4 time-step minima
  // adjoint: record cotangents, same layout as the records
  double* recbar = nullptr;
  size_t recbar_cap = 0;  // doubles
};

namespace {

int cuda_fail(pc_mol_handle* h, cudaError_t e) {
  if (e == cudaSuccess) return PC_OK;
  if (h) h->last_error = (e == cudaErrorMemoryAllocation) ? PC_ERR_OUT_OF_MEMORY : PC_ERR_CUDA;
  return (e == cudaErrorMemoryAllocation) ? PC_ERR_OUT_OF_MEMORY : PC_ERR_CUDA;
}

// 1/x rounded toward zero, on the host (the device's rcp_q): the nearest
// reciprocal, stepped one ulp toward zero where it exceeds 1/x in magnitude
// (r x > 1, decided exactly by the fused remainder).
double rcp_rz_host(double x) {
  double r = 1.0 / x;
  if (std::isfinite(r) && r != 0.0 && std::fma(r, x, -1.0) > 0.0) r = std::nextafter(r, 0.0);
  return r;
}

template <int NS>
void fill_common(DevMech<NS>& d, const pc_mechanism& m) {
  for (int k = 0; k < NS; ++k) {
    d.rW[k] = RU / m.mw[k];
    d.irW[k] = rcp_rz_host(d.rW[k]);
  }
  d.gamma = m.gamma;
  d.gm1 = m.gamma - 1.0;
  for (int k = 0; k < NS; ++k) d.cpk[k] = m.gamma / (m.gamma - 1.0) * RU / m.mw[k];
  d.const_mu = m.const_mu;
  d.const_xi = m.const_xi;
  d.const_lam = m.const_lambda;
  d.const_rhoD = m.const_rhoD;
}

template <int NS>
int fill_idealmix(DevMech<NS>& d, const pc_mechanism& m) {
  d.tmid = m.nasa_tmid[0];
  for (int k = 0; k < NS; ++k) {
    if (m.nasa_tmid[k] != d.tmid) return PC_ERR_UNSUPPORTED;  // one shared range split
    const double r = RU / m.mw[k];
    for (int n = 0; n < 6; ++n) {
      d.cpc[0][n][k] = r * m.nasa_lo[k][n];
      d.cpc[1][n][k] = r * m.nasa_hi[k][n];
    }
  }
  return PC_OK;
}

template <int NS>
int fill_simple(DevMech<NS>& d, const pc_mechanism& m) {
  for (int k = 0; k < NS; ++k) {
    for (int n = 0; n < 4; ++n) {
      d.visc[k][n] = m.visc_fit[k][n];
      d.cond[k][n] = m.cond_fit[k][n];
    }
    d.bulk[k] = m.bulk_ratio[k];
  }
  int q = 0;
  for (int k = 0; k < NS; ++k)
    for (int j = k + 1; j < NS; ++j, ++q)
      for (int n = 0; n < 4; ++n) {
        if (m.diff_fit[k][j][n] != m.diff_fit[j][k][n]) return PC_ERR_UNSUPPORTED;  // symmetric fits only
        d.diff[q][n] = m.diff_fit[k][j][n];
      }
  if (!(m.diff_pref > 0.0)) return PC_ERR_INVALID_ARGUMENT;
  d.inv_pref = 1.0 / m.diff_pref;
  return PC_OK;
}

// The species count whose kernels serve c (0: none compiled): one species
// with the GammaLaw EOS and constant transport, or 9 or 21 species with the
// ideal-gas mixture and mixture-averaged transport.
int compiled_variant(const pc_mol_config& c) {
  if (c.nspec == 1 && c.eos == PC_EOS_GAMMA_LAW && c.transport == PC_TRANSPORT_CONSTANT) return 1;
  if ((c.nspec == 9 || c.nspec == 21) && c.eos == PC_EOS_IDEAL_MIX && c.transport == PC_TRANSPORT_SIMPLE)
    return c.nspec;
  return 0;
}

// The device tables of the species count nspec from m; *nrec: doubles per record.
int fill_mechanism(MechSet& ms, int nspec, const pc_mechanism& m, int* nrec) {
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    DevMech<NS>& d = ms.get<NS>();
    fill_common(d, m);
    *nrec = Rec<NS>::N;
    if constexpr (NS == 1) return (int)PC_OK;
    int rc = fill_idealmix(d, m);
    if (rc == PC_OK) rc = fill_simple(d, m);
    return rc;
  });
}

bool covers(const pc_array4& a, const int lo[3], const int hi[3], int ng) {
  for (int d = 0; d < 3; ++d)
    if (a.begin[d] > lo[d] - ng || a.end[d] - 1 < hi[d] + ng) return false;
  return true;
}

int validate_box(const pc_box_desc& b, int nvar) {
  for (int d = 0; d < 3; ++d)
    if (b.hi[d] < b.lo[d]) return PC_ERR_INVALID_ARGUMENT;
  if (!b.state.p || !b.rhs.p) return PC_ERR_INVALID_ARGUMENT;
  if (b.state.ncomp < nvar || b.rhs.ncomp < nvar) return PC_ERR_INVALID_ARGUMENT;
  if (!covers(b.state, b.lo, b.hi, 2) || !covers(b.rhs, b.lo, b.hi, 0)) return PC_ERR_INVALID_ARGUMENT;
  const pc_array4* arrs[2] = {&b.state, &b.rhs};
  for (const pc_array4* a : arrs) {
    const long long nx = a->end[0] - a->begin[0], ny = a->end[1] - a->begin[1], nz = a->end[2] - a->begin[2];
    if (a->jstride < nx || a->kstride < a->jstride * ny || a->nstride < a->kstride * nz) return PC_ERR_INVALID_ARGUMENT;
  }
  // Cells of grow(valid, 2) are indexed with 32-bit chunk offsets.
  long long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    if (b.hi[d] - b.lo[d] + 1 > 4096) return PC_ERR_TOO_LARGE;
    ncell *= (long long)(b.hi[d] - b.lo[d] + 5);
  }
  if (ncell > 2000000000LL) return PC_ERR_TOO_LARGE;
  return PC_OK;
}

void build_layout(const pc_box_desc* boxes, int nboxes, int nrec, int tile, Layout& L) {
  const int TX = tile_extent(tile, 0), TY = tile_extent(tile, 1), TZ = tile_extent(tile, 2);
  L.boxes.clear();
  L.items.clear();
  L.tiles.clear();
  L.item_start.clear();
  L.tile_start.clear();
  L.scratch_doubles = 0;
  for (int bi = 0; bi < nboxes; ++bi) {
    const pc_box_desc& b = boxes[bi];
    DevBox d{};
    for (int a = 0; a < 3; ++a) {
      d.lo[a] = b.lo[a];
      d.hi[a] = b.hi[a];
      d.sb[a] = b.state.begin[a];
      d.rb[a] = b.rhs.begin[a];
      d.g2lo[a] = b.lo[a] - 2;
      d.n2[a] = b.hi[a] - b.lo[a] + 5;
    }
    d.S = b.state.p;
    d.sj = b.state.jstride;
    d.sk = b.state.kstride;
    d.sn = b.state.nstride;
    d.R = b.rhs.p;
    d.rj = b.rhs.jstride;
    d.rk = b.rhs.kstride;
    d.rn = b.rhs.nstride;
    d.ncell = (long long)d.n2[0] * d.n2[1] * d.n2[2];
    d.rec = reinterpret_cast<double*>(L.scratch_doubles);  // offset, rebased after allocation
    L.scratch_doubles += (size_t)d.ncell * nrec;
    L.scratch_doubles = (L.scratch_doubles + 31) & ~size_t(31);  // 256-byte aligned records
    L.boxes.push_back(d);
    L.item_start.push_back((int)L.items.size());
    for (long long c = 0; c < d.ncell; c += kCellThreads) L.items.push_back(make_int2(bi, (int)c));
    L.tile_start.push_back((int)L.tiles.size());
    // each column of tiles bottom to top: a persistent CTA's run of tiles
    // then hands its z face and slope layers from one tile to the next
    for (int j = b.lo[1]; j <= b.hi[1]; j += TY)
      for (int i = b.lo[0]; i <= b.hi[0]; i += TX)
        for (int k = b.lo[2]; k <= b.hi[2]; k += TZ) L.tiles.push_back(make_int4(bi, i, j, k));
  }
  L.item_start.push_back((int)L.items.size());
  L.tile_start.push_back((int)L.tiles.size());
}

template <class T>
int ensure(pc_mol_handle* h, T*& ptr, size_t& cap, size_t n) {
  if (n <= cap) return PC_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(h, e);
  cap = n;
  return PC_OK;
}

// Autotune key of a BoxArray: its multiset of box extents (the box-size
// histogram); the handle fixes the species count and the precision.
std::vector<int> tune_key(const pc_box_desc* boxes, int nboxes) {
  std::vector<int> k;
  k.reserve(3 * (size_t)nboxes);
  std::vector<long long> ext(nboxes);
  for (int b = 0; b < nboxes; ++b) {
    long long e = 0;
    for (int d = 2; d >= 0; --d) e = e * 8192 + (boxes[b].hi[d] - boxes[b].lo[d] + 1);
    ext[b] = e;
  }
  std::sort(ext.begin(), ext.end());
  for (long long e : ext) {
    k.push_back((int)(e % 8192));
    k.push_back((int)((e / 8192) % 8192));
    k.push_back((int)(e / (8192LL * 8192)));
  }
  return k;
}

bool is_mixed(int precision) { return precision == PC_PRECISION_MIXED || precision == PC_PRECISION_MIXED_FP64; }

// Dynamic shared memory of the flux pass at launch configuration t for the
// handle's species count and precision (bytes).  The FP64 passes stage one
// direction's face fluxes, cell slopes and the z carry; the mixed pass the
// face fluxes of all three directions.
size_t flux_pass_smem(const pc_mol_handle* h, int t) {
  return with_species(h->cfg.nspec, [&](auto sc) -> size_t {
    constexpr int NS = decltype(sc)::value;
    auto of = [&](auto tl) -> size_t {
      using TL = decltype(tl);
      if (is_mixed(h->cfg.precision)) return mixed_flux_smem_bytes<NS, TL>();
      return flux_smem_bytes<NS, TL>();
    };
    switch (t % kNumTiles) {
      case 1: return of(TileCube{});
      case 2: return of(TileLong{});
      case 3: return of(TileSmall{});
      default: return of(TileDefault{});
    }
  });
}

// Launch configuration t fits the device at the handle's species count: with
// 21 species the FP64 flux pass of the 8x8x8 and 16x8x4 tiles needs 278 and
// 343 KB of shared memory per CTA, more than the 227 KB a CTA may have.
bool config_fits(const pc_mol_handle* h, int t) { return flux_pass_smem(h, t) <= (size_t)h->smem_optin; }

int choose_tile(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes) {
  if (h->tile_forced >= 0) return h->tile_forced;
  if (h->tune_cache.empty()) return 0;
  auto it = h->tune_cache.find(tune_key(boxes, nboxes));
  return it == h->tune_cache.end() ? 0 : it->second;
}

// Everything of a box descriptor but its two array pointers.
bool same_geometry(const pc_box_desc& a, const pc_box_desc& b) {
  pc_box_desc x = a, y = b;
  x.state.p = y.state.p = nullptr;
  x.rhs.p = y.rhs.p = nullptr;
  return std::memcmp(&x, &y, sizeof(pc_box_desc)) == 0;
}

int prepare(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], cudaStream_t s) {
  const int nvar = 7 + h->cfg.nspec;
  for (int b = 0; b < nboxes; ++b) {
    int rc = validate_box(boxes[b], nvar);
    if (rc != PC_OK) return rc;
  }
  bool same_geom = (int)h->last_boxes.size() == nboxes && h->last_dx[0] == dx[0] && h->last_dx[1] == dx[1] &&
                   h->last_dx[2] == dx[2];
  for (int b = 0; same_geom && b < nboxes; ++b) same_geom = same_geometry(h->last_boxes[b], boxes[b]);
  if (h->tile_forced >= 0)
    h->tile = h->tile_forced;
  else if (!same_geom)
    h->tile = choose_tile(h, boxes, nboxes);
  int rc = PC_OK;
  const int shape = h->tile % kNumTiles;
  if (!(same_geom && h->lay_tile == shape)) {
    // New geometry: launch lists and record scratch.
    h->lay_tile = -1;
    build_layout(boxes, nboxes, h->nrec, shape, h->lay);
    rc = ensure(h, h->scratch, h->scratch_cap, h->lay.scratch_doubles);
    if (rc != PC_OK) return rc;
    for (auto& d : h->lay.boxes) d.rec = h->scratch + reinterpret_cast<size_t>(d.rec);
    if ((rc = ensure(h, h->d_items, h->cap_items, h->lay.items.size())) != PC_OK) return rc;
    if ((rc = ensure(h, h->d_tiles, h->cap_tiles, h->lay.tiles.size())) != PC_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(h->d_items, h->lay.items.data(), sizeof(int2) * h->lay.items.size(),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->d_tiles, h->lay.tiles.data(), sizeof(int4) * h->lay.tiles.size(),
                          cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(h, e);
    // The uploads above read host vectors owned by the handle; a layout
    // change waits for them before the vectors can be rebuilt.
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(h, e);
    for (auto& t : h->tables) t.key.clear();  // their record pointers are stale
    h->d_boxes = nullptr;
    h->last_boxes.assign(boxes, boxes + nboxes);
    for (int d = 0; d < 3; ++d) h->last_dx[d] = dx[d];
    h->lay_tile = shape;
  }
  // The device box table for these array pointers.
  pc_mol_handle::BoxTable* tb = nullptr;
  for (auto& t : h->tables)
    if (t.dev && (int)t.key.size() == nboxes && std::memcmp(t.key.data(), boxes, sizeof(pc_box_desc) * nboxes) == 0)
      tb = &t;
  if (!tb) {
    tb = &h->tables[0];
    for (auto& t : h->tables)
      if (t.stamp < tb->stamp) tb = &t;
    tb->host = h->lay.boxes;
    for (int b = 0; b < nboxes; ++b) {
      tb->host[b].S = boxes[b].state.p;
      tb->host[b].R = boxes[b].rhs.p;
    }
    if ((rc = ensure(h, tb->dev, tb->cap, tb->host.size())) != PC_OK) return rc;
    // Pageable source: the call returns once the data is staged, so the
    // host vector may change afterwards; the copy is ordered on s.
    const cudaError_t e =
        cudaMemcpyAsync(tb->dev, tb->host.data(), sizeof(DevBox) * tb->host.size(), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(h, e);
    tb->key.assign(boxes, boxes + nboxes);
  }
  tb->stamp = ++h->table_clock;
  h->d_boxes = tb->dev;
  h->last_boxes.assign(boxes, boxes + nboxes);
  return PC_OK;
}

Geo make_geo(const double dx[3]) {
  Geo g;
  for (int d = 0; d < 3; ++d) {
    g.dxs[d] = dx[d];
    g.dxinv[d] = 1.0 / dx[d];
  }
  g.area[0] = dx[1] * dx[2];
  g.area[1] = dx[0] * dx[2];
  g.area[2] = dx[0] * dx[1];
  g.vol = dx[0] * dx[1] * dx[2];
  g.ivol = rcp_rz_host(g.vol);
  g.p_ref = 0.0;
  return g;
}

template <int NS, class EOS, class TR>
int launch(pc_mol_handle* h, const DevMech<NS>& mech, const Geo& g, int ibeg, int iend, int tbeg, int tend,
           cudaStream_t s, bool timed, const FluxBox* fx) {
  if (timed) cudaEventRecord(h->ev[0], s);
  if (iend > ibeg) {
    const cudaError_t e = launch_cell_fp64<NS, EOS, TR>(h->d_boxes, h->d_items + ibeg, (unsigned)(iend - ibeg), mech,
                                                        h->flags, h->d_counters, s);
    if (e != cudaSuccess) return cuda_fail(h, e);
  }
  if (timed) cudaEventRecord(h->ev[1], s);
  const bool pers = h->tile >= kNumTiles;
  cudaError_t e = (h->lay_tile != 0)
                      ? launch_flux_fp64_tile(h->lay_tile, pers, h->variant, h->d_boxes, h->d_tiles + tbeg, tend - tbeg,
                                              h->mech, h->flags, g, h->d_counters, s, fx)
                      : launch_flux_fp64<NS, EOS>(h->d_boxes, h->d_tiles + tbeg, tend - tbeg, mech, h->flags, g,
                                                  h->d_counters, s, fx, pers);
  if (e == cudaSuccess)
    e = launch_flux_exact<NS, EOS>(h->d_boxes, h->d_tiles + tbeg, tend - tbeg, mech, h->flags, g, h->d_counters, s,
                                   fx);
  if (timed) cudaEventRecord(h->ev[2], s);
  return cuda_fail(h, e);
}

int run(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], void* stream, bool per_box,
        const FluxBox* fx = nullptr) {
  if (!h) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes < 0 || (nboxes > 0 && !boxes) || !dx) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0) || !std::isfinite(dx[d])) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  h->last_stream = s;
  rc = cuda_fail(h, cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * kNumCounters, s));
  if (rc != PC_OK) return rc;
  if (nboxes == 0) return h->last_error = PC_OK;
  rc = prepare(h, boxes, nboxes, dx, s);
  if (rc != PC_OK) return h->last_error = rc;
  const Geo g = make_geo(dx);
  const Layout& L = h->lay;
  const bool timed = h->cfg.time_passes != 0 && !per_box;
  h->timed = timed;
  const bool mixed = is_mixed(h->cfg.precision);
  const bool rcp = h->cfg.precision == PC_PRECISION_FP64_RCP;
  auto go = [&](int ib, int ie, int tb, int te) {
    if (rcp) {
      RcpLaunch a{};
      a.variant = h->variant;
      a.tile = h->lay_tile;
      a.persistent = h->tile >= kNumTiles;
      a.boxes = h->d_boxes;
      a.items = h->d_items + ib;
      a.nitems = ie - ib;
      a.tiles = h->d_tiles + tb;
      a.ntiles = te - tb;
      with_species(h->variant, [&](auto ns) {
        constexpr int NS = decltype(ns)::value;
        a.mech = &h->mech.get<NS>();
        a.mech_size = sizeof(DevMech<NS>);
        return 0;
      });
      a.flags = &h->flags;
      a.flags_size = sizeof h->flags;
      a.geo = &g;
      a.geo_size = sizeof g;
      a.fluxes = fx;
      a.fluxbox_size = sizeof(FluxBox);
      a.devbox_size = sizeof(DevBox);
      a.counters = h->d_counters;
      a.stream = s;
      for (int k = 0; k < 3; ++k) a.ev[k] = timed ? h->ev[k] : nullptr;
      return cuda_fail(h, launch_rhs_rcp(a));
    }
    if (mixed) {
      const double p_ref = h->cfg.mixed_p_ref > 0.0 ? h->cfg.mixed_p_ref : 1013250.0;
      Geo gm = g;
      gm.p_ref = p_ref;
      const int rc = launch_mixed(h->variant, h->lay_tile, h->tile >= kNumTiles,
                                  h->cfg.precision == PC_PRECISION_MIXED_FP64, h->d_boxes, h->d_items + ib, ie - ib,
                                  h->d_tiles + tb, te - tb, h->mech, h->flags, gm, p_ref, h->d_counters, s,
                                  timed ? h->ev[0] : nullptr, timed ? h->ev[1] : nullptr, timed ? h->ev[2] : nullptr,
                                  fx);
      return rc == 0 ? PC_OK : cuda_fail(h, cudaGetLastError());
    }
    return with_species(h->variant, [&](auto ns) {
      constexpr int NS = decltype(ns)::value;
      using P = Physics<NS>;
      return launch<NS, typename P::EOS, typename P::TR>(h, h->mech.get<NS>(), g, ib, ie, tb, te, s, timed, fx);
    });
  };
  if (!per_box) {
    rc = go(0, (int)L.items.size(), 0, (int)L.tiles.size());
  } else {
    for (int b = 0; b < nboxes && rc == PC_OK; ++b)
      rc = go(L.item_start[b], L.item_start[b + 1], L.tile_start[b], L.tile_start[b + 1]);
  }
  return h->last_error = rc;
}

}  // namespace

extern "C" {

int pc_mol_abi_version(void) { return PC_MOL_ABI_VERSION; }

const char* pc_mol_error_string(int code) {
  switch (code) {
    case PC_OK: return "ok";
    case PC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PC_ERR_UNSUPPORTED: return "unsupported configuration";
    case PC_ERR_CUDA: return "CUDA runtime error";
    case PC_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PC_ERR_NO_DEVICE: return "no CUDA device";
    case PC_ERR_TOO_LARGE: return "request exceeds a fixed-size limit";
    default: return "unknown status code";
  }
}

int pc_mol_create(pc_mol_handle** out, const pc_mol_config* cfg) {
  if (!out || !cfg) return PC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const pc_mol_config& c = *cfg;
  if (c.nspec != c.mech.nspec) return PC_ERR_INVALID_ARGUMENT;
  if (c.precision != PC_PRECISION_FP64 && !is_mixed(c.precision) && c.precision != PC_PRECISION_FP64_RCP)
    return PC_ERR_INVALID_ARGUMENT;
  const int variant = compiled_variant(c);
  if (!variant) return PC_ERR_UNSUPPORTED;
  for (int k = 0; k < c.nspec; ++k)
    if (!(c.mech.mw[k] > 0.0)) return PC_ERR_INVALID_ARGUMENT;
  if (c.eos == PC_EOS_GAMMA_LAW && !(c.mech.gamma > 1.0)) return PC_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PC_ERR_NO_DEVICE;
  pc_mol_handle* h = new (std::nothrow) pc_mol_handle();
  if (!h) return PC_ERR_OUT_OF_MEMORY;
  h->cfg = c;
  h->variant = variant;
  cudaGetDevice(&h->device);
  cudaDeviceGetAttribute(&h->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  const int rc = fill_mechanism(h->mech, variant, c.mech, &h->nrec);
  if (rc != PC_OK) {
    delete h;
    return rc;
  }
  h->flags.do_hydro = c.do_hydro != 0;
  h->flags.diffuse_vel = c.diffuse_vel != 0;
  h->flags.diffuse_temp = c.diffuse_temp != 0;
  h->flags.diffuse_spec = c.diffuse_spec != 0;
  h->flags.diffuse_enth = c.diffuse_enth != 0;
  h->flags.slopes = c.plm_iorder != 1;
  h->flags.laxf = c.use_laxf_flux != 0;
  h->flags.harmonic = c.transport_harmonic_mean != 0;
  h->flags.check_output = c.check_output != 0;
  h->flags.newton_maxit = c.newton_max_iter > 0 ? c.newton_max_iter : 50;
  if (cudaMalloc(&h->d_counters, sizeof(unsigned long long) * kNumCounters) != cudaSuccess) {
    delete h;
    return PC_ERR_OUT_OF_MEMORY;
  }
  cudaMemset(h->d_counters, 0, sizeof(unsigned long long) * kNumCounters);
  if (c.time_passes)
    for (auto& e : h->ev)
      if (cudaEventCreate(&e) != cudaSuccess) {
        pc_mol_destroy(h);
        return PC_ERR_CUDA;
      }
  *out = h;
  return PC_OK;
}

void pc_mol_destroy(pc_mol_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  cudaFree(h->d_counters);
  for (auto& t : h->tables) cudaFree(t.dev);
  cudaFree(h->d_items);
  cudaFree(h->d_tiles);
  cudaFree(h->scratch);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  for (auto& u : h->up) cudaFree(u.dev);
  cudaFree(h->d_dt);
  cudaFree(h->recbar);
  delete h;
}

int pc_mol_rhs_level(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], void* stream) {
  return run(h, boxes, nboxes, dx, stream, false);
}

int pc_mol_rhs_level_per_box(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                             void* stream) {
  return run(h, boxes, nboxes, dx, stream, true);
}

int pc_mol_last_status(pc_mol_handle* h, pc_mol_status* st) {
  if (!h || !st) return PC_ERR_INVALID_ARGUMENT;
  std::memset(st, 0, sizeof(*st));
  unsigned long long c[kNumCounters] = {};
  cudaError_t e = cudaSetDevice(h->device);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->last_stream);
  if (e == cudaSuccess) e = cudaMemcpy(c, h->d_counters, sizeof(c), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(h, e);
  st->cells = (long long)c[kCounterCells];
  st->newton_nonconverged = (long long)c[kCounterNewton];
  st->nonpositive_state = (long long)c[kCounterNonpos];
  st->nonfinite_output = (long long)c[kCounterNonfinite];
  st->exact_recomputes = (long long)(c[kCounterSlowCell] + c[kCounterSlowFlux] + c[kCounterSlowAdj]);
  st->last_error = h->last_error;
  return PC_OK;
}

int pc_mol_pass_times(pc_mol_handle* h, double* ms, int n) {
  if (!h || !ms || n < 2) return PC_ERR_INVALID_ARGUMENT;
  if (!h->cfg.time_passes || !h->timed) return PC_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaSetDevice(h->device);
  if (e == cudaSuccess) e = cudaEventSynchronize(h->ev[2]);
  float a = 0.f, b = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
  if (e != cudaSuccess) return cuda_fail(h, e);
  ms[0] = a;
  ms[1] = b;
  return PC_OK;
}

int pc_mol_tile_shape(int t, int shape[4]) {
  if (t < 0 || t >= kNumLaunchConfigs || !shape) return PC_ERR_INVALID_ARGUMENT;
  shape[0] = tile_extent(t % kNumTiles, 0);
  shape[1] = tile_extent(t % kNumTiles, 1);
  shape[2] = tile_extent(t % kNumTiles, 2);
  shape[3] = shape[0] * shape[1] * shape[2];
  return PC_OK;
}

int pc_mol_set_tile(pc_mol_handle* h, int t) {
  if (!h || t < -1 || t >= kNumLaunchConfigs) return PC_ERR_INVALID_ARGUMENT;
  if (t >= 0 && !config_fits(h, t)) return PC_ERR_UNSUPPORTED;
  h->tile_forced = t;
  h->last_boxes.clear();  // the next call chooses again
  return PC_OK;
}

int pc_mol_current_tile(pc_mol_handle* h, int* t) {
  if (!h || !t) return PC_ERR_INVALID_ARGUMENT;
  // h->tile, unless a call since (the tangent) ran at another shape
  *t = (h->lay_tile < 0 || h->lay_tile == h->tile % kNumTiles) ? h->tile : h->lay_tile;
  return PC_OK;
}

int pc_mol_autotune(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], int reps, int* best,
                    double* ms, int n_ms, void* stream) {
  if (!h || !best || nboxes <= 0 || !boxes || reps <= 0) return PC_ERR_INVALID_ARGUMENT;
  if (ms && n_ms < kNumLaunchConfigs) return PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return h->last_error = PC_ERR_CUDA;
  }
  const int saved = h->tile_forced;
  double tbest = 0.0;
  int ibest = 0;
  bool any = false;
  for (int t = 0; t < kNumLaunchConfigs && rc == PC_OK; ++t) {
    if (!config_fits(h, t)) {  // not timed
      if (ms) ms[t] = -1.0;
      continue;
    }
    h->tile_forced = t;
    rc = run(h, boxes, nboxes, dx, stream, false);  // warm-up, builds the layout of configuration t
    if (rc == PC_OK) rc = cuda_fail(h, cudaEventRecord(e0, s));
    for (int r = 0; r < reps && rc == PC_OK; ++r) rc = run(h, boxes, nboxes, dx, stream, false);
    if (rc == PC_OK) rc = cuda_fail(h, cudaEventRecord(e1, s));
    if (rc == PC_OK) rc = cuda_fail(h, cudaEventSynchronize(e1));
    float el = 0.f;
    if (rc == PC_OK) rc = cuda_fail(h, cudaEventElapsedTime(&el, e0, e1));
    const double per = (double)el / reps;
    if (ms) ms[t] = per;
    if (rc == PC_OK && (!any || per < tbest)) {
      tbest = per;
      ibest = t;
      any = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->tile_forced = saved;
  h->last_boxes.clear();
  if (rc != PC_OK) return h->last_error = rc;
  h->tune_cache[tune_key(boxes, nboxes)] = ibest;
  *best = ibest;
  return h->last_error = PC_OK;
}

}  // extern "C"

namespace {
__global__ void check_quotients_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                       double* __restrict__ q, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double bi = b[i];
    q[i] = div_by(a[i], bi, rcp_q(bi));
  }
}
}  // namespace

extern "C" int pc_mol_check_quotients(const double* a, const double* b, double* q, long long n, void* stream) {
  if (n < 0 || (n > 0 && (!a || !b || !q))) return PC_ERR_INVALID_ARGUMENT;
  if (n == 0) return PC_OK;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
  check_quotients_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(a, b, q, n);
  return cudaGetLastError() == cudaSuccess ? PC_OK : PC_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Single-box right-hand side that allocates no device memory.
//
// For callers that cannot call cudaMalloc while they run: code driven by an
// external memory pool that forbids other allocations, or an application
// that reserves all device memory up front.  The per-cell records, the
// launch lists and the diagnostic counters of one box live in
// g_static_scratch, a fixed array that the CUDA runtime reserves when this
// library is loaded and that every device holds until the process exits.
// The kernels are the ones pc_mol_rhs_level launches.  The first call on a
// device does the one-time set-up (the array's device address, the flux
// kernels' shared-memory opt-in); later calls make no such runtime call.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr size_t kStaticScratchBytes = size_t(48) << 20;  // 48 MiB
constexpr int kStaticMaxDevices = 64;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices] = {};

// Device address of g_static_scratch on the current device.  Host code may
// not use the symbol itself (it names a host-side shadow), so the address is
// looked up once per device, with that device current, and cached.
int static_scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PC_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kStaticMaxDevices) return PC_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return PC_ERR_CUDA;
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return PC_OK;
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// Writes the box table, the pass-1 chunk list and the pass-2 tile list of one
// box into the static array and clears the counters.
__global__ void static_lists_kernel(DevBox b, int nitems, int ntiles, int tiles_x, int tiles_y, DevBox* box_out,
                                    int2* items, int4* tiles, unsigned long long* counters) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    *box_out = b;
    for (int c = 0; c < kNumCounters; ++c) counters[c] = 0ull;
  }
  if (t < nitems) items[t] = make_int2(0, (int)(t * kCellThreads));
  if (t < ntiles) {
    const int tx = (int)(t % tiles_x), ty = (int)((t / tiles_x) % tiles_y), tz = (int)(t / ((long long)tiles_x * tiles_y));
    tiles[t] = make_int4(0, b.lo[0] + tx * kTX, b.lo[1] + ty * kTY, b.lo[2] + tz * kTZ);
  }
}

}  // namespace

extern "C" int pc_mol_rhs_box_static(const pc_mol_config* cfg, const pc_box_desc* box, const double dx[3],
                                     void* stream) {
  if (!cfg || !box || !dx) return PC_ERR_INVALID_ARGUMENT;
  const pc_mol_config& c = *cfg;
  if (c.nspec != c.mech.nspec) return PC_ERR_INVALID_ARGUMENT;
  if (c.precision != PC_PRECISION_FP64 && !is_mixed(c.precision)) return PC_ERR_UNSUPPORTED;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0) || !std::isfinite(dx[d])) return PC_ERR_INVALID_ARGUMENT;
  const int variant = compiled_variant(c);
  if (!variant) return PC_ERR_UNSUPPORTED;
  for (int k = 0; k < c.nspec; ++k)
    if (!(c.mech.mw[k] > 0.0)) return PC_ERR_INVALID_ARGUMENT;
  if (c.eos == PC_EOS_GAMMA_LAW && !(c.mech.gamma > 1.0)) return PC_ERR_INVALID_ARGUMENT;
  const int nvar = 7 + c.nspec;
  int rc = validate_box(*box, nvar);
  if (rc != PC_OK) return rc;

  MechSet ms{};
  int nrec = 0;
  rc = fill_mechanism(ms, variant, c.mech, &nrec);
  if (rc != PC_OK) return rc;
  DevFlags fl{};
  fl.do_hydro = c.do_hydro != 0;
  fl.diffuse_vel = c.diffuse_vel != 0;
  fl.diffuse_temp = c.diffuse_temp != 0;
  fl.diffuse_spec = c.diffuse_spec != 0;
  fl.diffuse_enth = c.diffuse_enth != 0;
  fl.slopes = c.plm_iorder != 1;
  fl.laxf = c.use_laxf_flux != 0;
  fl.harmonic = c.transport_harmonic_mean != 0;
  fl.check_output = c.check_output != 0;
  fl.newton_maxit = c.newton_max_iter > 0 ? c.newton_max_iter : 50;

  // Sections of the static array: counters | box | chunk list | tile list | records.
  int n2[3], nt[3];
  long long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    n2[d] = box->hi[d] - box->lo[d] + 5;
    ncell *= n2[d];
  }
  nt[0] = (box->hi[0] - box->lo[0] + kTX) / kTX;
  nt[1] = (box->hi[1] - box->lo[1] + kTY) / kTY;
  nt[2] = (box->hi[2] - box->lo[2] + kTZ) / kTZ;
  const long long nitems = (ncell + kCellThreads - 1) / kCellThreads;
  const long long ntiles = (long long)nt[0] * nt[1] * nt[2];
  const size_t off_ctr = 0;
  const size_t off_box = align256(off_ctr + sizeof(unsigned long long) * kNumCounters);
  const size_t off_items = align256(off_box + sizeof(DevBox));
  const size_t off_tiles = align256(off_items + sizeof(int2) * (size_t)nitems);
  const size_t off_rec = align256(off_tiles + sizeof(int4) * (size_t)ntiles);
  const size_t need = off_rec + sizeof(double) * (size_t)ncell * nrec;
  if (need > kStaticScratchBytes) return PC_ERR_TOO_LARGE;

  void* basev = nullptr;
  rc = static_scratch_address(&basev);
  if (rc != PC_OK) return rc;
  unsigned char* base = static_cast<unsigned char*>(basev);
  DevBox d{};
  for (int a = 0; a < 3; ++a) {
    d.lo[a] = box->lo[a];
    d.hi[a] = box->hi[a];
    d.sb[a] = box->state.begin[a];
    d.rb[a] = box->rhs.begin[a];
    d.g2lo[a] = box->lo[a] - 2;
    d.n2[a] = n2[a];
  }
  d.S = box->state.p;
  d.sj = box->state.jstride;
  d.sk = box->state.kstride;
  d.sn = box->state.nstride;
  d.R = box->rhs.p;
  d.rj = box->rhs.jstride;
  d.rk = box->rhs.kstride;
  d.rn = box->rhs.nstride;
  d.ncell = ncell;
  d.rec = reinterpret_cast<double*>(base + off_rec);
  DevBox* dbox = reinterpret_cast<DevBox*>(base + off_box);
  int2* items = reinterpret_cast<int2*>(base + off_items);
  int4* tiles = reinterpret_cast<int4*>(base + off_tiles);
  unsigned long long* ctr = reinterpret_cast<unsigned long long*>(base + off_ctr);

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long nlist = nitems > ntiles ? nitems : ntiles;
  static_lists_kernel<<<(unsigned)((nlist + 255) / 256), 256, 0, s>>>(d, (int)nitems, (int)ntiles, nt[0], nt[1], dbox,
                                                                       items, tiles, ctr);
  const Geo g = make_geo(dx);
  if (is_mixed(c.precision)) {  // the mixed passes on the same lists and scratch (its records are smaller)
    const double p_ref = c.mixed_p_ref > 0.0 ? c.mixed_p_ref : 1013250.0;
    Geo gm = g;
    gm.p_ref = p_ref;
    const int r = launch_mixed(variant, 0, false, c.precision == PC_PRECISION_MIXED_FP64, dbox, items, (int)nitems,
                               tiles, (int)ntiles, ms, fl, gm, p_ref, ctr, s, nullptr, nullptr, nullptr, nullptr);
    return r == 0 && cudaGetLastError() == cudaSuccess ? PC_OK : PC_ERR_CUDA;
  }
  const bool ok = with_species(variant, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    using P = Physics<NS>;
    const DevMech<NS>& m = ms.get<NS>();
    return launch_cell_fp64<NS, typename P::EOS, typename P::TR>(dbox, items, (unsigned)nitems, m, fl, ctr, s) ==
               cudaSuccess &&
           launch_flux_fp64<NS, typename P::EOS>(dbox, tiles, (int)ntiles, m, fl, g, ctr, s) == cudaSuccess &&
           launch_flux_exact<NS, typename P::EOS>(dbox, tiles, (int)ntiles, m, fl, g, ctr, s) == cudaSuccess;
  });
  if (!ok) return PC_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? PC_OK : PC_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Level operations of the MOL advance: ghost fill, LinComb, computeTemp and
// the time-step estimate (pc_level.cuh).
// ---------------------------------------------------------------------------
namespace {

enum {
  kUpFillBoxes = 0,
  kUpFillItems,
  kUpOwner,
  kUpLcDst,
  kUpLcX,
  kUpLcY,
  kUpItems,
  kUpBoxes,
  kUpAdjBoxes,
  kUpAdjFaces,
  kUpAdjOff,
  kUpFluxes
};

// Copies bytes to the handle's device slot unless they equal the last upload
// of that slot (repeated calls on the same layout launch kernels only).
int upload(pc_mol_handle* h, int slot, const void* data, size_t bytes, cudaStream_t s, void** dev) {
  pc_mol_handle::Upload& u = h->up[slot];
  if (bytes == 0) {
    *dev = u.dev;
    return PC_OK;
  }
  if (u.host.size() == bytes && u.dev && std::memcmp(u.host.data(), data, bytes) == 0) {
    *dev = u.dev;
    return PC_OK;
  }
  if (bytes > u.cap) {
    if (u.dev) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_fail(h, e);
      cudaFree(u.dev);
    }
    u.dev = nullptr;
    u.cap = 0;
    cudaError_t e = cudaMalloc(&u.dev, bytes);
    if (e != cudaSuccess) return cuda_fail(h, e);
    u.cap = bytes;
  }
  u.host.assign(static_cast<const unsigned char*>(data), static_cast<const unsigned char*>(data) + bytes);
  cudaError_t e = cudaMemcpyAsync(u.dev, u.host.data(), bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e);
  *dev = u.dev;
  return PC_OK;
}

LevelBox level_box(const int lo[3], const int hi[3], const pc_array4& a) {
  LevelBox b{};
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = lo[d];
    b.hi[d] = hi[d];
    b.sb[d] = a.begin[d];
  }
  b.S = a.p;
  b.sj = a.jstride;
  b.sk = a.kstride;
  b.sn = a.nstride;
  return b;
}

bool array_ok(const pc_array4& a, const int lo[3], const int hi[3], int ng, int nvar) {
  if (!a.p || a.ncomp < nvar) return false;
  for (int d = 0; d < 3; ++d)
    if (hi[d] < lo[d] || a.begin[d] > lo[d] - ng || a.end[d] - 1 < hi[d] + ng) return false;
  const long long nx = a.end[0] - a.begin[0], ny = a.end[1] - a.begin[1], nz = a.end[2] - a.begin[2];
  return a.jstride >= nx && a.kstride >= a.jstride * ny && a.nstride >= a.kstride * nz;
}

void chunk_items(const std::vector<long long>& ncells, std::vector<int2>& items) {
  items.clear();
  for (size_t b = 0; b < ncells.size(); ++b)
    for (long long c = 0; c < ncells[b]; c += 256) items.push_back(make_int2((int)b, (int)c));
}

long long nvalid(const int lo[3], const int hi[3], int ng) {
  long long n = 1;
  for (int d = 0; d < 3; ++d) n *= (long long)(hi[d] - lo[d] + 1 + 2 * ng);
  return n;
}

}  // namespace

static int fill_ghosts_impl(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const pc_geometry* geom,
                            int ngrow, void* stream, bool adjoint) {
  if (!h || !geom || nboxes < 0 || (nboxes > 0 && !boxes) || ngrow < 0) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes == 0 || ngrow == 0) return PC_OK;
  const int nvar = 7 + h->cfg.nspec;
  FillGeom g{};
  long long ndom = 1;
  for (int d = 0; d < 3; ++d) {
    g.dlo[d] = geom->domain_lo[d];
    g.dhi[d] = geom->domain_hi[d];
    g.len[d] = geom->domain_hi[d] - geom->domain_lo[d] + 1;
    g.bclo[d] = geom->bc_lo[d];
    g.bchi[d] = geom->bc_hi[d];
    if (g.len[d] < ngrow) return PC_ERR_INVALID_ARGUMENT;
    for (int bc : {geom->bc_lo[d], geom->bc_hi[d]})
      if (bc < PC_BC_INTERIOR || bc > PC_BC_NOSLIPWALL) return PC_ERR_UNSUPPORTED;
    if ((geom->bc_lo[d] == PC_BC_INTERIOR) != (geom->bc_hi[d] == PC_BC_INTERIOR)) return PC_ERR_INVALID_ARGUMENT;
    g.periodic[d] = geom->bc_lo[d] == PC_BC_INTERIOR;
    ndom *= g.len[d];
  }
  g.ng = ngrow;
  g.nvar = nvar;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  std::vector<LevelBox> lb;
  std::vector<long long> nc;
  for (int b = 0; b < nboxes; ++b) {
    if (!array_ok(boxes[b].state, boxes[b].lo, boxes[b].hi, ngrow, nvar)) return h->last_error = PC_ERR_INVALID_ARGUMENT;
    for (int d = 0; d < 3; ++d)
      if (boxes[b].lo[d] < g.dlo[d] || boxes[b].hi[d] > g.dhi[d]) return h->last_error = PC_ERR_INVALID_ARGUMENT;
    lb.push_back(level_box(boxes[b].lo, boxes[b].hi, boxes[b].state));
    nc.push_back(nvalid(boxes[b].lo, boxes[b].hi, ngrow));
  }
  std::vector<int2> items;
  chunk_items(nc, items);
  // Owner of each domain cell (several boxes): the valid boxes must tile the domain.
  void *dbox = nullptr, *ditems = nullptr, *downer = nullptr;
  if (nboxes > 1) {
    if (ndom > 400000000LL) return h->last_error = PC_ERR_TOO_LARGE;
    std::vector<int> owner((size_t)ndom, -1);
    for (int b = 0; b < nboxes; ++b)
      for (int k = boxes[b].lo[2]; k <= boxes[b].hi[2]; ++k)
        for (int j = boxes[b].lo[1]; j <= boxes[b].hi[1]; ++j)
          for (int i = boxes[b].lo[0]; i <= boxes[b].hi[0]; ++i) {
            const long long o = (i - g.dlo[0]) + (long long)(j - g.dlo[1]) * g.len[0] +
                                (long long)(k - g.dlo[2]) * g.len[0] * g.len[1];
            if (owner[o] >= 0) return h->last_error = PC_ERR_INVALID_ARGUMENT;  // overlapping boxes
            owner[o] = b;
          }
    for (int o : owner)
      if (o < 0) return h->last_error = PC_ERR_INVALID_ARGUMENT;  // domain not covered
    if ((rc = upload(h, kUpOwner, owner.data(), owner.size() * sizeof(int), s, &downer)) != PC_OK) return rc;
  } else {
    for (int d = 0; d < 3; ++d)
      if (boxes[0].lo[d] != g.dlo[d] || boxes[0].hi[d] != g.dhi[d]) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  }
  if ((rc = upload(h, kUpFillBoxes, lb.data(), lb.size() * sizeof(LevelBox), s, &dbox)) != PC_OK) return rc;
  if ((rc = upload(h, kUpFillItems, items.data(), items.size() * sizeof(int2), s, &ditems)) != PC_OK) return rc;
  if (adjoint)
    fill_ghosts_kernel<true><<<(unsigned)items.size(), 256, 0, s>>>(static_cast<const LevelBox*>(dbox),
                                                            static_cast<const int2*>(ditems),
                                                            nboxes > 1 ? static_cast<const int*>(downer) : nullptr, g);
  else
    fill_ghosts_kernel<false><<<(unsigned)items.size(), 256, 0, s>>>(static_cast<const LevelBox*>(dbox),
                                                            static_cast<const int2*>(ditems),
                                                            nboxes > 1 ? static_cast<const int*>(downer) : nullptr, g);
  return h->last_error = cuda_fail(h, cudaGetLastError());
}

extern "C" int pc_mol_fill_ghosts(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const pc_geometry* geom,
                                  int ngrow, void* stream) {
  return fill_ghosts_impl(h, boxes, nboxes, geom, ngrow, stream, false);
}

extern "C" int pc_mol_fill_ghosts_adjoint(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes,
                                          const pc_geometry* geom, int ngrow, void* stream) {
  return fill_ghosts_impl(h, boxes, nboxes, geom, ngrow, stream, true);
}

extern "C" int pc_mol_lincomb(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* dst, double a,
                              const pc_array4* x, double b, const pc_array4* y, void* stream) {
  if (!h || nboxes < 0 || (nboxes > 0 && (!lohi || !dst || !x || !y))) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes == 0) return PC_OK;
  const int nvar = 7 + h->cfg.nspec;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  std::vector<LevelBox> ld, lx, ly;
  std::vector<long long> nc;
  for (int i = 0; i < nboxes; ++i) {
    const int* lo = lohi + 6 * i;
    const int* hi = lohi + 6 * i + 3;
    if (!array_ok(dst[i], lo, hi, 0, nvar) || !array_ok(x[i], lo, hi, 0, nvar) || !array_ok(y[i], lo, hi, 0, nvar))
      return h->last_error = PC_ERR_INVALID_ARGUMENT;
    ld.push_back(level_box(lo, hi, dst[i]));
    lx.push_back(level_box(lo, hi, x[i]));
    ly.push_back(level_box(lo, hi, y[i]));
    nc.push_back(nvalid(lo, hi, 0));
  }
  std::vector<int2> items;
  chunk_items(nc, items);
  void *dd, *dx, *dy, *di;
  if ((rc = upload(h, kUpLcDst, ld.data(), ld.size() * sizeof(LevelBox), s, &dd)) != PC_OK) return rc;
  if ((rc = upload(h, kUpLcX, lx.data(), lx.size() * sizeof(LevelBox), s, &dx)) != PC_OK) return rc;
  if ((rc = upload(h, kUpLcY, ly.data(), ly.size() * sizeof(LevelBox), s, &dy)) != PC_OK) return rc;
  if ((rc = upload(h, kUpItems, items.data(), items.size() * sizeof(int2), s, &di)) != PC_OK) return rc;
  LinCombArgs A{static_cast<const LevelBox*>(dd), static_cast<const LevelBox*>(dx), static_cast<const LevelBox*>(dy),
                a, b, nvar};
  lincomb_kernel<<<(unsigned)items.size(), 256, 0, s>>>(static_cast<const int2*>(di), A);
  return h->last_error = cuda_fail(h, cudaGetLastError());
}

extern "C" int pc_mol_compute_temp(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* state,
                                   void* stream) {
  if (!h || nboxes < 0 || (nboxes > 0 && (!lohi || !state))) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes == 0) return PC_OK;
  const int nvar = 7 + h->cfg.nspec;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  std::vector<LevelBox> lb;
  std::vector<long long> nc;
  for (int i = 0; i < nboxes; ++i) {
    const int* lo = lohi + 6 * i;
    const int* hi = lohi + 6 * i + 3;
    if (!array_ok(state[i], lo, hi, 0, nvar)) return h->last_error = PC_ERR_INVALID_ARGUMENT;
    lb.push_back(level_box(lo, hi, state[i]));
    nc.push_back(nvalid(lo, hi, 0));
  }
  std::vector<int2> items;
  chunk_items(nc, items);
  void *db, *di;
  if ((rc = upload(h, kUpBoxes, lb.data(), lb.size() * sizeof(LevelBox), s, &db)) != PC_OK) return rc;
  if ((rc = upload(h, kUpItems, items.data(), items.size() * sizeof(int2), s, &di)) != PC_OK) return rc;
  h->last_stream = s;
  cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * kNumCounters, s);
  const int maxit = h->flags.newton_maxit;
  with_species(h->variant, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    compute_temp_kernel<NS, typename Physics<NS>::EOS><<<(unsigned)items.size(), 256, 0, s>>>(
        static_cast<const LevelBox*>(db), static_cast<const int2*>(di), h->mech.get<NS>(), maxit, h->d_counters);
    return 0;
  });
  return h->last_error = cuda_fail(h, cudaGetLastError());
}

extern "C" int pc_mol_compute_temp_adjoint(pc_mol_handle* h, int nboxes, const int* lohi, const pc_array4* state,
                                           pc_array4* state_bar, void* stream) {
  if (!h || nboxes < 0 || (nboxes > 0 && (!lohi || !state || !state_bar))) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes == 0) return PC_OK;
  const int nvar = 7 + h->cfg.nspec;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  std::vector<LevelBox> lb, lq;
  std::vector<long long> nc;
  for (int i = 0; i < nboxes; ++i) {
    const int* lo = lohi + 6 * i;
    const int* hi = lohi + 6 * i + 3;
    if (!array_ok(state[i], lo, hi, 0, nvar) || !array_ok(state_bar[i], lo, hi, 0, nvar))
      return h->last_error = PC_ERR_INVALID_ARGUMENT;
    lb.push_back(level_box(lo, hi, state[i]));
    lq.push_back(level_box(lo, hi, state_bar[i]));
    nc.push_back(nvalid(lo, hi, 0));
  }
  std::vector<int2> items;
  chunk_items(nc, items);
  void *db, *dq, *di;
  if ((rc = upload(h, kUpBoxes, lb.data(), lb.size() * sizeof(LevelBox), s, &db)) != PC_OK) return rc;
  if ((rc = upload(h, kUpLcDst, lq.data(), lq.size() * sizeof(LevelBox), s, &dq)) != PC_OK) return rc;
  if ((rc = upload(h, kUpItems, items.data(), items.size() * sizeof(int2), s, &di)) != PC_OK) return rc;
  h->last_stream = s;
  with_species(h->variant, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    compute_temp_adjoint_kernel<NS, typename Physics<NS>::EOS><<<(unsigned)items.size(), 256, 0, s>>>(
        static_cast<const LevelBox*>(db), static_cast<const LevelBox*>(dq), static_cast<const int2*>(di),
        h->mech.get<NS>());
    return 0;
  });
  return h->last_error = cuda_fail(h, cudaGetLastError());
}

extern "C" int pc_mol_est_dt(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3], double cfl,
                             double max_dt, double* dt, void* stream) {
  if (!h || !dx || !dt || nboxes < 0 || (nboxes > 0 && !boxes) || !(cfl > 0.0) || !(max_dt > 0.0))
    return PC_ERR_INVALID_ARGUMENT;
  const int nvar = 7 + h->cfg.nspec;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  if (!h->d_dt && (rc = cuda_fail(h, cudaMalloc(&h->d_dt, 4 * sizeof(unsigned long long)))) != PC_OK) return rc;
  std::vector<LevelBox> lb;
  std::vector<long long> nc;
  for (int i = 0; i < nboxes; ++i) {
    if (!array_ok(boxes[i].state, boxes[i].lo, boxes[i].hi, 0, nvar)) return h->last_error = PC_ERR_INVALID_ARGUMENT;
    lb.push_back(level_box(boxes[i].lo, boxes[i].hi, boxes[i].state));
    nc.push_back(nvalid(boxes[i].lo, boxes[i].hi, 0));
  }
  std::vector<int2> items;
  chunk_items(nc, items);
  const unsigned long long inf[4] = {0x7ff0000000000000ull, 0x7ff0000000000000ull, 0x7ff0000000000000ull,
                                     0x7ff0000000000000ull};
  cudaError_t e = cudaMemcpyAsync(h->d_dt, inf, sizeof(inf), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e);
  if (!items.empty()) {
    void *db, *di;
    if ((rc = upload(h, kUpBoxes, lb.data(), lb.size() * sizeof(LevelBox), s, &db)) != PC_OK) return rc;
    if ((rc = upload(h, kUpItems, items.data(), items.size() * sizeof(int2), s, &di)) != PC_OK) return rc;
    const Geo g = make_geo(dx);
    with_species(h->variant, [&](auto ns) {
      constexpr int NS = decltype(ns)::value;
      using P = Physics<NS>;
      est_dt_kernel<NS, typename P::EOS, typename P::TR><<<(unsigned)items.size(), 256, 0, s>>>(
          static_cast<const LevelBox*>(db), static_cast<const int2*>(di), h->mech.get<NS>(), g, h->d_dt);
      return 0;
    });
  }
  unsigned long long bits[4];
  e = cudaMemcpyAsync(bits, h->d_dt, sizeof(bits), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e);
  double m4[4];
  std::memcpy(m4, bits, sizeof(m4));
  const double mdc = max_dt / cfl;
  double eh = mdc, ev = mdc, et = mdc, ee = mdc;
  if (h->cfg.do_hydro) eh = std::min(eh, m4[0]);
  if (h->cfg.diffuse_vel) ev = std::min(ev, m4[1]);
  if (h->cfg.diffuse_temp) et = std::min(et, m4[2]);
  if (h->cfg.diffuse_enth) ee = std::min(ee, m4[3]);
  eh = std::min(eh, std::min(ev, std::min(et, ee)));
  eh *= cfl;
  *dt = std::min(max_dt, eh);
  return h->last_error = PC_OK;
}

// ---------------------------------------------------------------------------
// Vector-Jacobian product of the RHS (pc_adjoint.cuh).
// ---------------------------------------------------------------------------
extern "C" int pc_mol_rhs_vjp(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                              const pc_array4* rhs_bar, pc_array4* state_bar, void* stream) {
  if (!h) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes < 0 || (nboxes > 0 && (!boxes || !rhs_bar || !state_bar)) || !dx)
    return h->last_error = PC_ERR_INVALID_ARGUMENT;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0) || !std::isfinite(dx[d])) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  if (h->cfg.precision != PC_PRECISION_FP64 || h->flags.laxf) return h->last_error = PC_ERR_UNSUPPORTED;
  const int nvar = 7 + h->cfg.nspec;
  for (int b = 0; b < nboxes; ++b)
    if (!array_ok(rhs_bar[b], boxes[b].lo, boxes[b].hi, 0, nvar) ||
        !array_ok(state_bar[b], boxes[b].lo, boxes[b].hi, 2, nvar))
      return h->last_error = PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  h->last_stream = s;
  rc = cuda_fail(h, cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * kNumCounters, s));
  if (rc != PC_OK) return rc;
  if (nboxes == 0) return h->last_error = PC_OK;
  if ((rc = prepare(h, boxes, nboxes, dx, s)) != PC_OK) return h->last_error = rc;
  const Layout& L = h->lay;
  // per-box cotangent arrays, face chunks, record offsets
  std::vector<AdjBox> adj(nboxes);
  std::vector<int4> fitems;
  std::vector<long long> off(nboxes);
  for (int b = 0; b < nboxes; ++b) {
    AdjBox& a = adj[b];
    const pc_array4 &r = rhs_bar[b], &u = state_bar[b];
    a.rbar = r.p;
    a.rj = r.jstride;
    a.rk = r.kstride;
    a.rn = r.nstride;
    a.ubar = u.p;
    a.uj = u.jstride;
    a.uk = u.kstride;
    a.un = u.nstride;
    for (int d = 0; d < 3; ++d) {
      a.rb[d] = r.begin[d];
      a.ub[d] = u.begin[d];
    }
    off[b] = (long long)(L.boxes[b].rec - h->scratch);
    const int n0 = boxes[b].hi[0] - boxes[b].lo[0] + 1, n1 = boxes[b].hi[1] - boxes[b].lo[1] + 1,
              n2 = boxes[b].hi[2] - boxes[b].lo[2] + 1;
    for (int d = 0; d < 3; ++d) {
      const long long nf = (long long)(n0 + (d == 0)) * (n1 + (d == 1)) * (n2 + (d == 2));
      for (long long c = 0; c * kAdjThreads < nf; ++c) fitems.push_back(make_int4(b, d, (int)c, 0));
    }
  }
  if ((rc = ensure(h, h->recbar, h->recbar_cap, L.scratch_doubles)) != PC_OK) return h->last_error = rc;
  void *dadj = nullptr, *dfit = nullptr, *doff = nullptr;
  if ((rc = upload(h, kUpAdjBoxes, adj.data(), adj.size() * sizeof(AdjBox), s, &dadj)) != PC_OK) return rc;
  if ((rc = upload(h, kUpAdjFaces, fitems.data(), fitems.size() * sizeof(int4), s, &dfit)) != PC_OK) return rc;
  if ((rc = upload(h, kUpAdjOff, off.data(), off.size() * sizeof(long long), s, &doff)) != PC_OK) return rc;
  // pass 1: records of the forward state
  const int nitems = (int)L.items.size();
  const cudaError_t ec = with_species(h->variant, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    using P = Physics<NS>;
    return launch_cell_fp64<NS, typename P::EOS, typename P::TR>(h->d_boxes, h->d_items, (unsigned)nitems,
                                                                 h->mech.get<NS>(), h->flags, h->d_counters, s);
  });
  if ((rc = cuda_fail(h, ec)) != PC_OK) return rc;
  if ((rc = cuda_fail(h, cudaMemsetAsync(h->recbar, 0, sizeof(double) * L.scratch_doubles, s))) != PC_OK) return rc;
  const cudaError_t e = launch_vjp_passes(h->variant, h->d_boxes, static_cast<const AdjBox*>(dadj), h->d_items, nitems,
                                          static_cast<const int4*>(dfit), (int)fitems.size(), h->recbar,
                                          (long long)L.scratch_doubles, static_cast<const long long*>(doff),
                                          h->mech, h->flags, make_geo(dx), h->d_counters, s);
  return h->last_error = cuda_fail(h, e);
}

// ---------------------------------------------------------------------------
// RHS with the face fluxes exported (refluxing).
// ---------------------------------------------------------------------------
extern "C" int pc_mol_rhs_level_fluxes(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                                       const pc_array4* fluxes, void* stream) {
  if (!h) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes < 0 || (nboxes > 0 && (!boxes || !fluxes))) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  const int nvar = 7 + h->cfg.nspec;
  std::vector<FluxBox> fb(nboxes);
  for (int b = 0; b < nboxes; ++b) {
    for (int d = 0; d < 3; ++d) {
      int hi[3] = {boxes[b].hi[0], boxes[b].hi[1], boxes[b].hi[2]};
      hi[d] += 1;  // surroundingNodes(valid, d)
      const pc_array4& a = fluxes[3 * b + d];
      if (!array_ok(a, boxes[b].lo, hi, 0, nvar)) return h->last_error = PC_ERR_INVALID_ARGUMENT;
      fb[b].p[d] = a.p;
      fb[b].js[d] = a.jstride;
      fb[b].ks[d] = a.kstride;
      fb[b].ns[d] = a.nstride;
      for (int e = 0; e < 3; ++e) fb[b].b[d][e] = a.begin[e];
    }
  }
  if (nboxes == 0) return run(h, boxes, nboxes, dx, stream, false);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  void* dfx = nullptr;
  if ((rc = upload(h, kUpFluxes, fb.data(), fb.size() * sizeof(FluxBox), static_cast<cudaStream_t>(stream), &dfx)) !=
      PC_OK)
    return rc;
  return run(h, boxes, nboxes, dx, stream, false, static_cast<const FluxBox*>(dfx));
}

// ---------------------------------------------------------------------------
// Jacobian-vector product of the RHS (pc_tangent.cuh).
// ---------------------------------------------------------------------------
extern "C" int pc_mol_rhs_jvp(pc_mol_handle* h, const pc_box_desc* boxes, int nboxes, const double dx[3],
                              const pc_array4* state_dot, pc_array4* rhs_dot, void* stream) {
  if (!h) return PC_ERR_INVALID_ARGUMENT;
  if (nboxes < 0 || (nboxes > 0 && (!boxes || !state_dot || !rhs_dot)) || !dx)
    return h->last_error = PC_ERR_INVALID_ARGUMENT;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0) || !std::isfinite(dx[d])) return h->last_error = PC_ERR_INVALID_ARGUMENT;
  if (h->cfg.precision != PC_PRECISION_FP64) return h->last_error = PC_ERR_UNSUPPORTED;
  const int nvar = 7 + h->cfg.nspec;
  for (int b = 0; b < nboxes; ++b)
    if (!array_ok(state_dot[b], boxes[b].lo, boxes[b].hi, 2, nvar) ||
        !array_ok(rhs_dot[b], boxes[b].lo, boxes[b].hi, 0, nvar))
      return h->last_error = PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(h, cudaSetDevice(h->device));
  if (rc != PC_OK) return rc;
  h->last_stream = s;
  rc = cuda_fail(h, cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * kNumCounters, s));
  if (rc != PC_OK) return rc;
  if (nboxes == 0) return h->last_error = PC_OK;
  // The tangent flux pass runs on 8x4x4 tiles.
  const int saved_forced = h->tile_forced, saved_tile = h->tile;
  h->tile_forced = 3;
  rc = prepare(h, boxes, nboxes, dx, s);
  h->tile_forced = saved_forced;
  h->tile = (saved_forced >= 0 || rc != PC_OK) ? saved_tile : choose_tile(h, boxes, nboxes);
  if (rc != PC_OK) return h->last_error = rc;
  const Layout& L = h->lay;
  if ((rc = ensure(h, h->recbar, h->recbar_cap, L.scratch_doubles)) != PC_OK) return h->last_error = rc;
  std::vector<TanBox> tan(nboxes);
  for (int b = 0; b < nboxes; ++b) {
    TanBox& t = tan[b];
    const pc_array4 &sd = state_dot[b], &rd = rhs_dot[b];
    t.Sd = sd.p;
    t.sj = sd.jstride;
    t.sk = sd.kstride;
    t.sn = sd.nstride;
    t.Rd = rd.p;
    t.rj = rd.jstride;
    t.rk = rd.kstride;
    t.rn = rd.nstride;
    for (int d = 0; d < 3; ++d) {
      t.sb[d] = sd.begin[d];
      t.rb[d] = rd.begin[d];
    }
    t.trec = h->recbar + (L.boxes[b].rec - h->scratch);
  }
  void* dtan = nullptr;
  if ((rc = upload(h, kUpAdjBoxes, tan.data(), tan.size() * sizeof(TanBox), s, &dtan)) != PC_OK) return rc;
  const cudaError_t e = launch_jvp_passes(h->variant, h->d_boxes, static_cast<const TanBox*>(dtan), h->d_items,
                                          (int)L.items.size(), h->d_tiles, (int)L.tiles.size(), h->mech, h->flags,
                                          make_geo(dx), h->d_counters, s);
  return h->last_error = cuda_fail(h, e);
}

// ---------------------------------------------------------------------------
// CUDA graph of (ghost fill +) RHS.
// ---------------------------------------------------------------------------
struct pc_mol_graph {
  pc_mol_handle* h = nullptr;  // private handle: its layout, scratch and counters belong to the graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" int pc_mol_graph_create(pc_mol_handle* parent, const pc_box_desc* boxes, int nboxes, const double dx[3],
                                   const pc_geometry* fill_geom, int ngrow, pc_mol_graph** out) {
  if (!parent || !out || nboxes <= 0 || !boxes || !dx) return PC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int rc = cuda_fail(parent, cudaSetDevice(parent->device));
  if (rc != PC_OK) return rc;
  // The captured kernels read the box table, tile list and record scratch of
  // the handle they were launched through; a private handle keeps them alive
  // and unchanged for the graph's lifetime whatever the caller's handle does.
  pc_mol_config cfg = parent->cfg;
  cfg.time_passes = 0;
  pc_mol_graph* g = new (std::nothrow) pc_mol_graph();
  if (!g) return parent->last_error = PC_ERR_OUT_OF_MEMORY;
  rc = pc_mol_create(&g->h, &cfg);
  if (rc != PC_OK) {
    delete g;
    return parent->last_error = rc;
  }
  pc_mol_handle* h = g->h;
  h->tile_forced = parent->tile_forced;
  h->tune_cache = parent->tune_cache;
  cudaStream_t s = nullptr;
  rc = cuda_fail(h, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  auto seq = [&]() -> int {
    int r = PC_OK;
    if (fill_geom) r = pc_mol_fill_ghosts(h, boxes, nboxes, fill_geom, ngrow, s);
    if (r == PC_OK) r = run(h, boxes, nboxes, dx, s, false);
    return r;
  };
  // One uncaptured pass performs every upload and allocation.
  if (rc == PC_OK) rc = seq();
  if (rc == PC_OK) rc = cuda_fail(h, cudaStreamSynchronize(s));
  if (rc == PC_OK) rc = cuda_fail(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  if (rc == PC_OK) {
    const int r1 = seq();
    const cudaError_t e = cudaStreamEndCapture(s, &g->graph);
    rc = r1 != PC_OK ? r1 : cuda_fail(h, e);
  }
  if (rc == PC_OK) rc = cuda_fail(h, cudaGraphInstantiate(&g->exec, g->graph, 0));
  if (s) cudaStreamDestroy(s);
  if (rc != PC_OK) {
    pc_mol_graph_destroy(g);
    return parent->last_error = rc;
  }
  *out = g;
  return PC_OK;
}

extern "C" int pc_mol_graph_launch(pc_mol_graph* g, void* stream) {
  if (!g || !g->exec) return PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(g->h, cudaSetDevice(g->h->device));
  if (rc != PC_OK) return rc;
  g->h->last_stream = s;
  return g->h->last_error = cuda_fail(g->h, cudaGraphLaunch(g->exec, s));
}

extern "C" int pc_mol_graph_status(pc_mol_graph* g, pc_mol_status* st) {
  if (!g) return PC_ERR_INVALID_ARGUMENT;
  return pc_mol_last_status(g->h, st);
}

extern "C" void pc_mol_graph_destroy(pc_mol_graph* g) {
  if (!g) return;
  if (g->h) cudaSetDevice(g->h->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  pc_mol_destroy(g->h);
  delete g;
}

// ---------------------------------------------------------------------------
// One SSP-RK2 step of a level per CUDA-graph replay: do_mol_advance without
// sources (Source/Advance.cpp:98-168):
//   fill(S_old); R = RHS(S_old); S_new = 1 S_old + dt R; computeTemp(S_new)
//   fill(S_new); R = RHS(S_new); S_new = 0.5 S_new + 0.5 S_old;
//   S_new = 1 S_new + 0.5 dt R; computeTemp(S_new)
// Two graphs, A -> B and B -> A, share one private handle (RHS layout,
// record scratch, counters) and device tables built once at creation; the
// time step is a device scalar written by a one-thread kernel ahead of each
// replay, which the LinComb kernels read.
// ---------------------------------------------------------------------------
struct pc_mol_step_graph {
  pc_mol_handle* h = nullptr;
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  double* d_dt = nullptr;
  std::vector<void*> bufs;  // device tables owned by the graphs
};

namespace {

// A device buffer owned by g holding bytes copied from src (src null: left
// uninitialised).
int dev_copy(pc_mol_step_graph* g, const void* src, size_t bytes, void** out) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return PC_ERR_OUT_OF_MEMORY;
  g->bufs.push_back(p);
  if (src && bytes && cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return PC_ERR_CUDA;
  *out = p;
  return PC_OK;
}

}  // namespace

extern "C" void pc_mol_step_graph_destroy(pc_mol_step_graph* g) {
  if (!g) return;
  if (g->h) cudaSetDevice(g->h->device);
  for (int d = 0; d < 2; ++d) {
    if (g->exec[d]) cudaGraphExecDestroy(g->exec[d]);
    if (g->graph[d]) cudaGraphDestroy(g->graph[d]);
  }
  for (void* p : g->bufs) cudaFree(p);
  pc_mol_destroy(g->h);
  delete g;
}

extern "C" int pc_mol_step_graph_create(pc_mol_handle* parent, const pc_box_desc* a, const pc_array4* state_b,
                                        int nboxes, const double dx[3], const pc_geometry* geom, int ngrow,
                                        pc_mol_step_graph** out) {
  if (!parent || !out || nboxes <= 0 || !a || !state_b || !dx || !geom || ngrow < 2) return PC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const int nvar = 7 + parent->cfg.nspec;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0) || !std::isfinite(dx[d])) return parent->last_error = PC_ERR_INVALID_ARGUMENT;
  // Both states have the same array geometry (so the RHS layout is shared)
  // and at least ngrow filled ghost layers; the RHS array is the valid box.
  std::vector<pc_box_desc> da(a, a + nboxes), db(a, a + nboxes);
  for (int b = 0; b < nboxes; ++b) {
    db[b].state = state_b[b];
    if (!same_geometry(da[b], db[b]) || a[b].state.p == state_b[b].p ||
        !array_ok(a[b].state, a[b].lo, a[b].hi, ngrow, nvar) || !array_ok(a[b].rhs, a[b].lo, a[b].hi, 0, nvar))
      return parent->last_error = PC_ERR_INVALID_ARGUMENT;
  }
  int rc = cuda_fail(parent, cudaSetDevice(parent->device));
  if (rc != PC_OK) return rc;
  pc_mol_config cfg = parent->cfg;
  cfg.time_passes = 0;
  pc_mol_step_graph* g = new (std::nothrow) pc_mol_step_graph();
  if (!g) return parent->last_error = PC_ERR_OUT_OF_MEMORY;
  rc = pc_mol_create(&g->h, &cfg);
  if (rc != PC_OK) {
    delete g;
    return parent->last_error = rc;
  }
  pc_mol_handle* h = g->h;
  h->tile_forced = parent->tile_forced;
  h->tune_cache = parent->tune_cache;
  auto fail = [&](int r) {
    pc_mol_step_graph_destroy(g);
    return parent->last_error = r;
  };

  // Host tables: each state's and the RHS's LevelBox lists, the valid-cell
  // and grown-box chunk lists, the fill geometry and the owner map.
  FillGeom fg{};
  long long ndom = 1;
  for (int d = 0; d < 3; ++d) {
    fg.dlo[d] = geom->domain_lo[d];
    fg.dhi[d] = geom->domain_hi[d];
    fg.len[d] = geom->domain_hi[d] - geom->domain_lo[d] + 1;
    fg.bclo[d] = geom->bc_lo[d];
    fg.bchi[d] = geom->bc_hi[d];
    if (fg.len[d] < ngrow) return fail(PC_ERR_INVALID_ARGUMENT);
    for (int bc : {geom->bc_lo[d], geom->bc_hi[d]})
      if (bc < PC_BC_INTERIOR || bc > PC_BC_NOSLIPWALL) return fail(PC_ERR_UNSUPPORTED);
    if ((geom->bc_lo[d] == PC_BC_INTERIOR) != (geom->bc_hi[d] == PC_BC_INTERIOR)) return fail(PC_ERR_INVALID_ARGUMENT);
    fg.periodic[d] = geom->bc_lo[d] == PC_BC_INTERIOR;
    ndom *= fg.len[d];
  }
  fg.ng = ngrow;
  fg.nvar = nvar;
  std::vector<LevelBox> lbA, lbB, lbR;
  std::vector<long long> ncv, ncg;
  for (int b = 0; b < nboxes; ++b) {
    for (int d = 0; d < 3; ++d)
      if (a[b].lo[d] < fg.dlo[d] || a[b].hi[d] > fg.dhi[d]) return fail(PC_ERR_INVALID_ARGUMENT);
    lbA.push_back(level_box(a[b].lo, a[b].hi, a[b].state));
    lbB.push_back(level_box(a[b].lo, a[b].hi, state_b[b]));
    lbR.push_back(level_box(a[b].lo, a[b].hi, a[b].rhs));
    ncv.push_back(nvalid(a[b].lo, a[b].hi, 0));
    ncg.push_back(nvalid(a[b].lo, a[b].hi, ngrow));
  }
  std::vector<int2> itv, itg;
  chunk_items(ncv, itv);
  chunk_items(ncg, itg);
  std::vector<int> owner;
  if (nboxes > 1) {
    if (ndom > 400000000LL) return fail(PC_ERR_TOO_LARGE);
    owner.assign((size_t)ndom, -1);
    for (int b = 0; b < nboxes; ++b)
      for (int k = a[b].lo[2]; k <= a[b].hi[2]; ++k)
        for (int j = a[b].lo[1]; j <= a[b].hi[1]; ++j)
          for (int i = a[b].lo[0]; i <= a[b].hi[0]; ++i) {
            const long long o = (i - fg.dlo[0]) + (long long)(j - fg.dlo[1]) * fg.len[0] +
                                (long long)(k - fg.dlo[2]) * fg.len[0] * fg.len[1];
            if (owner[o] >= 0) return fail(PC_ERR_INVALID_ARGUMENT);
            owner[o] = b;
          }
    for (int o : owner)
      if (o < 0) return fail(PC_ERR_INVALID_ARGUMENT);
  } else {
    for (int d = 0; d < 3; ++d)
      if (a[0].lo[d] != fg.dlo[d] || a[0].hi[d] != fg.dhi[d]) return fail(PC_ERR_INVALID_ARGUMENT);
  }
  void *dA, *dB, *dR, *dItv, *dItg, *dOwn = nullptr, *dDt;
  if ((rc = dev_copy(g, lbA.data(), lbA.size() * sizeof(LevelBox), &dA)) != PC_OK ||
      (rc = dev_copy(g, lbB.data(), lbB.size() * sizeof(LevelBox), &dB)) != PC_OK ||
      (rc = dev_copy(g, lbR.data(), lbR.size() * sizeof(LevelBox), &dR)) != PC_OK ||
      (rc = dev_copy(g, itv.data(), itv.size() * sizeof(int2), &dItv)) != PC_OK ||
      (rc = dev_copy(g, itg.data(), itg.size() * sizeof(int2), &dItg)) != PC_OK ||
      (rc = dev_copy(g, nullptr, sizeof(double), &dDt)) != PC_OK)
    return fail(rc);
  if (!owner.empty() && (rc = dev_copy(g, owner.data(), owner.size() * sizeof(int), &dOwn)) != PC_OK) return fail(rc);
  g->d_dt = static_cast<double*>(dDt);

  cudaStream_t s = nullptr;
  rc = cuda_fail(h, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  if (rc != PC_OK) return fail(rc);
  const LevelBox* L[2] = {static_cast<const LevelBox*>(dA), static_cast<const LevelBox*>(dB)};
  const LevelBox* LR = static_cast<const LevelBox*>(dR);
  const int2* ITV = static_cast<const int2*>(dItv);
  const int2* ITG = static_cast<const int2*>(dItg);
  const int* OWN = static_cast<const int*>(dOwn);
  const std::vector<pc_box_desc>* D[2] = {&da, &db};
  const unsigned nbv = (unsigned)itv.size(), nbg = (unsigned)itg.size();
  const int maxit = h->flags.newton_maxit;
  auto ctemp = [&](const LevelBox* lb) {
    with_species(h->variant, [&](auto ns) {
      constexpr int NS = decltype(ns)::value;
      compute_temp_kernel<NS, typename Physics<NS>::EOS><<<nbv, 256, 0, s>>>(lb, ITV, h->mech.get<NS>(), maxit,
                                                                             h->d_counters);
      return 0;
    });
  };
  // The step from state o to state n (o, n = 0: A, 1: B).
  auto seq = [&](int o) -> int {
    const int n = 1 - o;
    fill_ghosts_kernel<false><<<nbg, 256, 0, s>>>(L[o], ITG, OWN, fg);
    int r = run(h, D[o]->data(), nboxes, dx, s, false);
    if (r != PC_OK) return r;
    lincomb_dt_kernel<<<nbv, 256, 0, s>>>(ITV, LinCombArgs{L[n], L[o], LR, 1.0, 1.0, nvar}, g->d_dt);
    ctemp(L[n]);
    fill_ghosts_kernel<false><<<nbg, 256, 0, s>>>(L[n], ITG, OWN, fg);
    r = run(h, D[n]->data(), nboxes, dx, s, false);
    if (r != PC_OK) return r;
    lincomb_kernel<<<nbv, 256, 0, s>>>(ITV, LinCombArgs{L[n], L[n], L[o], 0.5, 0.5, nvar});
    lincomb_dt_kernel<<<nbv, 256, 0, s>>>(ITV, LinCombArgs{L[n], L[n], LR, 1.0, 0.5, nvar}, g->d_dt);
    ctemp(L[n]);
    return cuda_fail(h, cudaGetLastError());
  };
  // Uncaptured RHS evaluations of both states make every upload and
  // allocation the captured RHS needs (the layout and the box tables of both
  // states); they write only R, whatever the states hold.
  for (int o = 0; o < 2 && rc == PC_OK; ++o) rc = run(h, D[o]->data(), nboxes, dx, s, false);
  if (rc == PC_OK) rc = cuda_fail(h, cudaStreamSynchronize(s));
  for (int o = 0; o < 2 && rc == PC_OK; ++o) {
    rc = cuda_fail(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    if (rc != PC_OK) break;
    const int r1 = seq(o);
    const cudaError_t e = cudaStreamEndCapture(s, &g->graph[o]);
    rc = r1 != PC_OK ? r1 : cuda_fail(h, e);
    if (rc == PC_OK) rc = cuda_fail(h, cudaGraphInstantiate(&g->exec[o], g->graph[o], 0));
  }
  if (s) cudaStreamDestroy(s);
  if (rc != PC_OK) return fail(rc);
  *out = g;
  return PC_OK;
}

extern "C" int pc_mol_step_graph_launch(pc_mol_step_graph* g, double dt, int reverse, void* stream) {
  if (!g || !g->exec[0] || !g->exec[1] || !(dt >= 0.0) || !std::isfinite(dt)) return PC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_fail(g->h, cudaSetDevice(g->h->device));
  if (rc != PC_OK) return rc;
  g->h->last_stream = s;
  set_scalar_kernel<<<1, 1, 0, s>>>(g->d_dt, dt);
  rc = cuda_fail(g->h, cudaGetLastError());
  if (rc != PC_OK) return g->h->last_error = rc;
  return g->h->last_error = cuda_fail(g->h, cudaGraphLaunch(g->exec[reverse ? 1 : 0], s));
}

extern "C" int pc_mol_step_graph_status(pc_mol_step_graph* g, pc_mol_status* st) {
  if (!g) return PC_ERR_INVALID_ARGUMENT;
  return pc_mol_last_status(g->h, st);
}

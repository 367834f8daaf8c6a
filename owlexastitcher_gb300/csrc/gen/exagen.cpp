// exagen.cpp -- synthetic AMR hierarchy and its ExaStitch dual mesh.
//
// Restates the reference's offline toolchain for in-memory use:
//   * the AMR input of tools/amrMakeDualMesh/makeDual.cpp (leaf cells with a
//     position in finest units and a level; level 0 is finest),
//   * makeDual.cpp:596-872 (doCell): every 2x2x2 block of neighbouring
//     cell centres forms a dual cell; uniform blocks become "perfect cubes",
//     the rest are classified into tets, pyramids, wedges and hexes,
//   * makeGrids.cpp:57-209: perfect cubes of one level are grouped by
//     8x8x8 macrocell into bricks ("gridlets") of vertex scalars,
//   * model/ExaStitchModel.cpp:24-257: element vertices carry their cell's
//     value, index rows are 8 wide padded with -1, absent gridlet vertices
//     are NaN, unused vertices are compacted away.
//
// The reference's find() (makeDual.cpp:172-195) searches sorted cell lists
// level by level; here the hierarchy is held as per-level "refined" and
// "leaf" bit sets with rank tables, so locating the leaf that contains a
// point is a short descent from the root.  Dual cells are generated once,
// by the lowest (y, x, z) cell of the finest level among their corners
// (makeDual.cpp:641-655), exactly as in the reference.
#include "exagen_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using exagen::Field;
using exagen::FieldView;
using exagen::Stream;

namespace {
thread_local std::string g_err;
} // namespace

namespace exagen {

void setLastError(const std::string &msg) { g_err = msg; }

int numThreadsOf(const exa_gen_params *p)
{
#ifdef _OPENMP
  return p->numThreads > 0 ? p->numThreads : omp_get_max_threads();
#else
  (void)p;
  return 1;
#endif
}

void checkParams(const exa_gen_params *p)
{
  if (!p) throw std::runtime_error("null argument");
  if (p->numLevels < 1 || p->numLevels > kMaxLevels) throw std::runtime_error("numLevels must be in [1,16]");
  for (int a = 0; a < 3; ++a)
    if (p->rootDims[a] < 1) throw std::runtime_error("rootDims must be positive");
  if (p->noiseOctaves < 0 || p->noiseOctaves > kMaxOctaves) throw std::runtime_error("noiseOctaves must be in [0,16]");
}

void Field::setup(const exa_gen_params &P)
{
  const int Lroot = P.numLevels - 1;
  kind = P.fieldKind;
  seed = P.seed;
  noiseAmp = P.noiseAmplitude;
  octaves = P.noiseOctaves;
  for (int a = 0; a < 3; ++a) extent[a] = (double)((int64_t)P.rootDims[a] << Lroot);
  // lattice values of each octave inside the unit cube, precomputed
  const FieldView v0 = view();
  latTab.assign(octaves, {});
  latN.assign(octaves, 0);
  double f = kind == EXA_FIELD_GAUSSIANS ? 4.0 : 2.0;
  for (int o = 0; o < octaves; ++o, f *= 2.0) {
    const int m = (int)f + 2;
    latN[o] = m;
    latTab[o].resize((size_t)m * m * m);
    for (int k = 0; k < m; ++k)
      for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) latTab[o][((size_t)k * m + j) * m + i] = (float)lattice(v0, i, j, k, o);
  }
  if (kind == EXA_FIELD_GAUSSIANS) {
    Stream s(P.seed);
    K = P.numGaussians;
    for (int k = 0; k < K; ++k) {
      cx.push_back(s.next01()); cy.push_back(s.next01()); cz.push_back(s.next01());
      sx.push_back(s.uniform(0.03, 0.15)); sy.push_back(s.uniform(0.03, 0.15));
      sz.push_back(s.uniform(0.03, 0.15));
      amp.push_back(s.uniform(0.2, 1.0));
    }
  }
}

FieldView Field::view() const
{
  FieldView v{};
  v.kind = kind;
  v.K = K;
  v.octaves = octaves;
  v.seed = seed;
  v.noiseAmp = noiseAmp;
  for (int a = 0; a < 3; ++a) v.extent[a] = extent[a];
  v.cloudLo = cloudLo;
  v.cloudHi = cloudHi;
  for (int o = 0; o < (int)latTab.size() && o < kMaxOctaves; ++o) {
    v.lat[o] = latTab[o].data();
    v.latN[o] = latN[o];
  }
  for (int a = 0; a < 3; ++a)
    for (int L = 0; L < (int)gtab[a].size() && L < kMaxLevels; ++L) v.gtab[a][L] = gtab[a][L].data();
  return v;
}

double Field::evalUnit(double x, double y, double z) const
{
  const FieldView v = view();
  if (kind == EXA_FIELD_CLOUD) return cloud_map(v, cloud_raw(v, x, y, z));
  double g = 0;
  for (int k = 0; k < K; ++k) g += amp[k] * gauss1(k, 0, x) * gauss1(k, 1, y) * gauss1(k, 2, z);
  return g + noiseAmp * octave_noise(v, x, y, z, 4.0, octaves);
}

} // namespace exagen

namespace {

// ---------------------------------------------------------------- bitsets
struct Bits {
  std::vector<uint64_t> w;
  std::vector<uint64_t> rank;  // prefix popcount per word
  void resize(uint64_t n) { w.assign((n + 63) / 64, 0); }
  bool get(uint64_t i) const { return (w[i >> 6] >> (i & 63)) & 1; }
  void set(uint64_t i) { w[i >> 6] |= (1ull << (i & 63)); }
  void setAtomic(uint64_t i)
  {
    __atomic_fetch_or(&w[i >> 6], 1ull << (i & 63), __ATOMIC_RELAXED);
  }
  void buildRank()
  {
    rank.resize(w.size() + 1);
    uint64_t acc = 0;
    for (size_t k = 0; k < w.size(); ++k) { rank[k] = acc; acc += (uint64_t)__builtin_popcountll(w[k]); }
    rank[w.size()] = acc;
  }
  uint64_t count() const { return rank.empty() ? 0 : rank.back(); }
  uint64_t rankOf(uint64_t i) const
  {
    const uint64_t word = w[i >> 6] & ((1ull << (i & 63)) - 1ull);
    return rank[i >> 6] + (uint64_t)__builtin_popcountll(word);
  }
};

struct Level {
  int64_t n[3];  // cells per axis
  Bits refined;  // cell exists and has children
  Bits leaf;     // cell exists and is a leaf
  uint64_t leafOffset = 0;
  uint64_t lin(int64_t i, int64_t j, int64_t k) const { return ((uint64_t)k * n[1] + j) * n[0] + i; }
  bool inside(int64_t i, int64_t j, int64_t k) const
  {
    return i >= 0 && j >= 0 && k >= 0 && i < n[0] && j < n[1] && k < n[2];
  }
};

struct LeafRef { int level; uint64_t lin; uint64_t id; };

struct Elem { int type; uint32_t v[8]; };  // type 0 tet, 1 pyr, 2 wedge, 3 hex; v = leaf ids

using exagen::numThreadsOf;

struct Builder {
  const exa_gen_params &P;
  exa_gen_result &R;
  int Lroot;
  std::vector<Level> lv;
  std::vector<float> value;  // per leaf id

  Builder(const exa_gen_params &p, exa_gen_result &r) : P(p), R(r)
  {
    Lroot = p.numLevels - 1;
    lv.resize(p.numLevels);
    for (int L = 0; L <= Lroot; ++L)
      for (int a = 0; a < 3; ++a) lv[L].n[a] = (int64_t)p.rootDims[a] << (Lroot - L);
  }

  double center(int L, int64_t i) const { return exagen::cell_center(L, i); }
  FieldView fv{};  // the field as the evaluations read it (after set-up)

  void buildGaussTables()
  {
    Field &F = R.field;
    for (int a = 0; a < 3; ++a) F.gtab[a].assign(lv.size(), {});
    if (F.kind == EXA_FIELD_GAUSSIANS) {
      for (int L = 0; L <= Lroot; ++L)
        for (int a = 0; a < 3; ++a) {
          const int64_t n = lv[L].n[a];
          auto &T = F.gtab[a][L];
          T.resize((size_t)n * F.K);
#pragma omp parallel for schedule(static) num_threads(numThreadsOf(&P))
          for (int64_t i = 0; i < n; ++i) F.gaussRow(a, L, i, &T[(size_t)i * F.K]);
        }
    }
    fv = F.view();
  }
  double evalCell(int L, int64_t i, int64_t j, int64_t k) const { return exagen::eval_cell(fv, L, i, j, k); }

  void setupField()
  {
    Field &F = R.field;
    F.setup(P);
    if (F.kind == EXA_FIELD_CLOUD) {
      // cloud: the mapping sends the requested fraction of root cells to 0
      const FieldView v = F.view();
      Level &R0 = lv[Lroot];
      const uint64_t n = (uint64_t)R0.n[0] * R0.n[1] * R0.n[2];
      std::vector<double> raw(n);
#pragma omp parallel for schedule(static) num_threads(numThreadsOf(&P))
      for (int64_t c = 0; c < (int64_t)n; ++c) {
        const int64_t i = c % R0.n[0], j = (c / R0.n[0]) % R0.n[1], k = c / (R0.n[0] * R0.n[1]);
        raw[c] = exagen::cloud_raw(v, center(Lroot, i) / F.extent[0], center(Lroot, j) / F.extent[1],
                                   center(Lroot, k) / F.extent[2]);
      }
      std::vector<double> sorted = raw;
      const size_t q = std::min(n - 1, (size_t)(P.cloudEmptyFraction * (double)n));
      std::nth_element(sorted.begin(), sorted.begin() + q, sorted.end());
      const double lo = sorted[q];
      const double hi = *std::max_element(raw.begin(), raw.end());
      F.cloudLo = lo;
      F.cloudHi = hi > lo ? hi : lo + 1.0;
    }
  }

  bool refineCrit(double v, int L, double maxAbs) const
  {
    return exagen::refine_crit(P.fieldKind, v, L, Lroot, (double)P.refineThreshold, maxAbs);
  }

  void buildTree()
  {
    const int nt = numThreadsOf(&P);
    for (int L = 1; L <= Lroot; ++L) {
      Level &l = lv[L];
      l.refined.resize((uint64_t)l.n[0] * l.n[1] * l.n[2]);
    }
    // root: max |f| over root-level centres defines the threshold scale
    Level &root = lv[Lroot];
    const uint64_t nRoot = (uint64_t)root.n[0] * root.n[1] * root.n[2];
    std::vector<float> rootVal(nRoot);
    double maxAbs = 0;
#pragma omp parallel for schedule(static) reduction(max : maxAbs) num_threads(nt)
    for (int64_t c = 0; c < (int64_t)nRoot; ++c) {
      const int64_t i = c % root.n[0], j = (c / root.n[0]) % root.n[1], k = c / (root.n[0] * root.n[1]);
      const double v = evalCell(Lroot, i, j, k);
      rootVal[c] = (float)v;
      maxAbs = std::max(maxAbs, std::fabs(v));
    }
    if (Lroot > 0) {
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int64_t c = 0; c < (int64_t)nRoot; ++c)
        if (refineCrit(rootVal[c], Lroot, maxAbs)) root.refined.setAtomic((uint64_t)c);
    }
    // top-down: children of refined cells
    for (int L = Lroot - 1; L >= 1; --L) {
      Level &par = lv[L + 1];
      Level &cur = lv[L];
      const int64_t nw = (int64_t)par.refined.w.size();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
      for (int64_t wi = 0; wi < nw; ++wi) {
        uint64_t word = par.refined.w[wi];
        while (word) {
          const int b = __builtin_ctzll(word);
          word &= word - 1;
          const uint64_t pc = (uint64_t)wi * 64 + b;
          const int64_t pi = pc % par.n[0], pj = (pc / par.n[0]) % par.n[1], pk = pc / (par.n[0] * par.n[1]);
          for (int d = 0; d < 8; ++d) {
            const int64_t i = 2 * pi + (d & 1), j = 2 * pj + ((d >> 1) & 1), k = 2 * pk + (d >> 2);
            if (refineCrit(evalCell(L, i, j, k), L, maxAbs)) cur.refined.setAtomic(cur.lin(i, j, k));
          }
        }
      }
    }
    if (P.balance) balance();
    // leaf sets and ids: levels ascending, then linear index
    uint64_t off = 0;
    for (int L = 0; L <= Lroot; ++L) {
      Level &l = lv[L];
      const uint64_t n = (uint64_t)l.n[0] * l.n[1] * l.n[2];
      l.leaf.resize(n);
      if (L == Lroot) {
        for (size_t k = 0; k < l.leaf.w.size(); ++k) {
          uint64_t all = ~0ull;
          if ((k + 1) * 64 > n) all = (n % 64) ? ((1ull << (n % 64)) - 1ull) : ~0ull;
          l.leaf.w[k] = all & ~(l.refined.w.empty() ? 0ull : l.refined.w[k]);
        }
      } else {
        const Level &par = lv[L + 1];
        const int64_t nw = (int64_t)par.refined.w.size();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
        for (int64_t wi = 0; wi < nw; ++wi) {
          uint64_t word = par.refined.w[wi];
          while (word) {
            const int b = __builtin_ctzll(word);
            word &= word - 1;
            const uint64_t pc = (uint64_t)wi * 64 + b;
            const int64_t pi = pc % par.n[0], pj = (pc / par.n[0]) % par.n[1], pk = pc / (par.n[0] * par.n[1]);
            for (int d = 0; d < 8; ++d) {
              const int64_t i = 2 * pi + (d & 1), j = 2 * pj + ((d >> 1) & 1), k = 2 * pk + (d >> 2);
              const uint64_t c = l.lin(i, j, k);
              if (L == 0 || !l.refined.get(c)) l.leaf.setAtomic(c);
            }
          }
        }
      }
      l.leaf.buildRank();
      l.leafOffset = off;
      off += l.leaf.count();
      R.stats.numCellsPerLevel[L] = l.leaf.count();
    }
    R.stats.numAmrCells = off;
  }

  // 2:1 balance: every same-level neighbour of a refined cell exists
  void balance()
  {
    for (int L = 1; L < Lroot; ++L) {
      Level &cur = lv[L];
      Level &par = lv[L + 1];
      const int64_t nw = (int64_t)cur.refined.w.size();
#pragma omp parallel for schedule(dynamic, 256) num_threads(numThreadsOf(&P))
      for (int64_t wi = 0; wi < nw; ++wi) {
        uint64_t word = cur.refined.w[wi];
        while (word) {
          const int b = __builtin_ctzll(word);
          word &= word - 1;
          const uint64_t c = (uint64_t)wi * 64 + b;
          const int64_t i = c % cur.n[0], j = (c / cur.n[0]) % cur.n[1], k = c / (cur.n[0] * cur.n[1]);
          for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
              for (int dx = -1; dx <= 1; ++dx) {
                const int64_t ni = i + dx, nj = j + dy, nk = k + dz;
                if (!cur.inside(ni, nj, nk)) continue;
                par.refined.setAtomic(par.lin(ni >> 1, nj >> 1, nk >> 1));
              }
        }
      }
    }
  }

  // leaf containing the point q (in half finest units), or level -1
  LeafRef findHalf(int64_t qx, int64_t qy, int64_t qz) const
  {
    LeafRef r{-1, 0, 0};
    if (qx < 0 || qy < 0 || qz < 0) return r;
    for (int L = Lroot; L >= 0; --L) {
      const Level &l = lv[L];
      const int sh = L + 1;
      const int64_t i = qx >> sh, j = qy >> sh, k = qz >> sh;
      if (!l.inside(i, j, k)) return r;
      const uint64_t c = l.lin(i, j, k);
      if (l.leaf.get(c)) { r.level = L; r.lin = c; r.id = l.leafOffset + l.leaf.rankOf(c); return r; }
      if (L == 0 || !l.refined.get(c)) return r;
    }
    return r;
  }

  void computeValues()
  {
    value.resize(R.stats.numAmrCells);
    R.amrCells.resize(R.stats.numAmrCells * 4);
    for (int L = 0; L <= Lroot; ++L) {
      const Level &l = lv[L];
      const int64_t nw = (int64_t)l.leaf.w.size();
#pragma omp parallel for schedule(dynamic, 256) num_threads(numThreadsOf(&P))
      for (int64_t wi = 0; wi < nw; ++wi) {
        uint64_t word = l.leaf.w[wi];
        uint64_t id = l.leafOffset + l.leaf.rank[wi];
        while (word) {
          const int b = __builtin_ctzll(word);
          word &= word - 1;
          const uint64_t c = (uint64_t)wi * 64 + b;
          const int64_t i = c % l.n[0], j = (c / l.n[0]) % l.n[1], k = c / (l.n[0] * l.n[1]);
          value[id] = (float)evalCell(L, i, j, k);
          int32_t *rec = &R.amrCells[id * 4];
          rec[0] = (int32_t)(i << L); rec[1] = (int32_t)(j << L); rec[2] = (int32_t)(k << L); rec[3] = L;
          id++;
        }
      }
    }
    R.amrScalars = value;
    float mn = INFINITY, mx = -INFINITY;
    for (float v : value) { mn = std::min(mn, v); mx = std::max(mx, v); }
    R.stats.fieldMin = mn; R.stats.fieldMax = mx;
  }

  // ---- makeDual.cpp:596-872 for the non-uniform dual cells ----
  // LogicalCell order of makeDual.cpp:115-122 for same-level cells with
  // non-negative positions: (pos.y, pos.x, pos.z)
  static bool cellLess(int64_t ai, int64_t aj, int64_t ak, int64_t bi, int64_t bj, int64_t bk)
  {
    if (aj != bj) return aj < bj;
    if (ai != bi) return ai < bi;
    return ak < bk;
  }

  void emitTet(std::vector<Elem> *out, uint64_t a, uint64_t b, uint64_t c, uint64_t d)
  {
    Elem e{0, {(uint32_t)a, (uint32_t)b, (uint32_t)c, (uint32_t)d, 0, 0, 0, 0}};
    out[0].push_back(e);
  }

  void doCell(int L, int64_t ci, int64_t cj, int64_t ck, std::vector<Elem> *out, uint64_t &skipped)
  {
    const Level &l = lv[L];
    // quick reject: all 26 same-level neighbours are leaves (or outside)
    bool uniform = true;
    for (int dz = -1; dz <= 1 && uniform; ++dz)
      for (int dy = -1; dy <= 1 && uniform; ++dy)
        for (int dx = -1; dx <= 1 && uniform; ++dx) {
          const int64_t i = ci + dx, j = cj + dy, k = ck + dz;
          if (!l.inside(i, j, k)) continue;
          if (!l.leaf.get(l.lin(i, j, k))) uniform = false;
        }
    if (uniform) return;
    LeafRef nb[27];
    const int64_t w = 1ll << L;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int64_t i = ci + dx, j = cj + dy, k = ck + dz;
          LeafRef &r = nb[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
          if (l.inside(i, j, k) && l.leaf.get(l.lin(i, j, k))) {
            const uint64_t c = l.lin(i, j, k);
            r = LeafRef{L, c, l.leafOffset + l.leaf.rankOf(c)};
          } else {
            // neighbour centre in half units: 2*(pos + d*w) + w
            r = findHalf(2 * i * w + w, 2 * j * w + w, 2 * k * w + w);
          }
        }
    const uint64_t selfId = nb[13].id;
    for (int dz = -1; dz <= 1; dz += 2)
      for (int dy = -1; dy <= 1; dy += 2)
        for (int dx = -1; dx <= 1; dx += 2) {
          LeafRef corner[2][2][2];
          int minLevel = 1000, maxLevel = -1, numFound = 0;
          for (int iz = 0; iz < 2; iz++)
            for (int iy = 0; iy < 2; iy++)
              for (int ix = 0; ix < 2; ix++) {
                const LeafRef &r = nb[(dz * iz + 1) * 9 + (dy * iy + 1) * 3 + (dx * ix + 1)];
                corner[iz][iy][ix] = r;
                if (r.level < 0) continue;
                minLevel = std::min(minLevel, r.level);
                maxLevel = std::max(maxLevel, r.level);
                ++numFound;
              }
          if (numFound < 8) continue;
          if (minLevel < L) continue;
          if (minLevel == maxLevel) continue;  // perfect cube: a gridlet cell
          // generated by the lowest same-level corner (makeDual.cpp:641-655)
          bool isMin = true;
          for (int iz = 0; iz < 2 && isMin; iz++)
            for (int iy = 0; iy < 2 && isMin; iy++)
              for (int ix = 0; ix < 2 && isMin; ix++) {
                const LeafRef &r = corner[iz][iy][ix];
                if (r.level != L || r.id == selfId) continue;
                const int64_t i = r.lin % l.n[0], j = (r.lin / l.n[0]) % l.n[1], k = r.lin / (l.n[0] * l.n[1]);
                if (cellLess(i, j, k, ci, cj, ck)) isMin = false;
              }
          if (!isMin) continue;
          uint64_t vtx[2][2][2];
          for (int iz = 0; iz < 2; iz++)
            for (int iy = 0; iy < 2; iy++)
              for (int ix = 0; ix < 2; ix++) vtx[iz][iy][ix] = corner[iz][iy][ix].id;
          if (dx < 0) { std::swap(vtx[0][0][0], vtx[0][0][1]); std::swap(vtx[0][1][0], vtx[0][1][1]);
                        std::swap(vtx[1][0][0], vtx[1][0][1]); std::swap(vtx[1][1][0], vtx[1][1][1]); }
          if (dy < 0) { std::swap(vtx[0][0][0], vtx[0][1][0]); std::swap(vtx[0][0][1], vtx[0][1][1]);
                        std::swap(vtx[1][0][0], vtx[1][1][0]); std::swap(vtx[1][0][1], vtx[1][1][1]); }
          if (dz < 0) { std::swap(vtx[0][0][0], vtx[1][0][0]); std::swap(vtx[0][0][1], vtx[1][0][1]);
                        std::swap(vtx[0][1][0], vtx[1][1][0]); std::swap(vtx[0][1][1], vtx[1][1][1]); }
          const uint64_t v[8] = {vtx[0][0][0], vtx[0][0][1], vtx[0][1][1], vtx[0][1][0],
                                 vtx[1][0][0], vtx[1][0][1], vtx[1][1][1], vtx[1][1][0]};
          uint64_t u[8];
          std::copy(v, v + 8, u);
          std::sort(u, u + 8);
          const int numUnique = (int)(std::unique(u, u + 8) - u);
          classify(v, numUnique, out, skipped);
        }
  }

  // makeDual.cpp:496-547
  void tryPyramid(const uint64_t base[4], uint64_t top, int numUnique, std::vector<Elem> *out, uint64_t &skipped)
  {
    if (numUnique == 5) {
      Elem e{1, {(uint32_t)base[0], (uint32_t)base[1], (uint32_t)base[2], (uint32_t)base[3], (uint32_t)top, 0, 0, 0}};
      out[1].push_back(e);
      return;
    }
    if (numUnique == 4) {
      if (base[0] == base[1]) { emitTet(out, base[1], base[2], base[3], top); return; }
      if (base[1] == base[2]) { emitTet(out, base[2], base[3], base[0], top); return; }
      if (base[2] == base[3]) { emitTet(out, base[3], base[0], base[1], top); return; }
      if (base[3] == base[0]) { emitTet(out, base[0], base[1], base[2], top); return; }
      if (base[0] == base[2] || base[1] == base[3]) { skipped++; return; }
    }
    // the reference throws here ("this case should not happen")
    skipped++;
  }

  void wedge(const uint64_t *v, int f0, int f1, int f2, int b0, int b1, int b2, std::vector<Elem> *out)
  {
    Elem e{2, {(uint32_t)v[f0], (uint32_t)v[f1], (uint32_t)v[f2], (uint32_t)v[b0], (uint32_t)v[b1], (uint32_t)v[b2], 0, 0}};
    out[2].push_back(e);
  }

  void hex(const uint64_t *v, std::vector<Elem> *out)
  {
    Elem e{3, {}};
    for (int i = 0; i < 8; ++i) e.v[i] = (uint32_t)v[i];
    out[3].push_back(e);
  }

  // makeDual.cpp:734-870, non-uniform dual cells only
  void classify(const uint64_t *v, int numUnique, std::vector<Elem> *out, uint64_t &skipped)
  {
    auto allSame = [&](int a, int b, int c, int d) { return v[a] == v[b] && v[a] == v[c] && v[a] == v[d]; };
    auto same = [&](int a, int b) { return v[a] == v[b]; };
    if (numUnique == 8) { hex(v, out); return; }
    if (numUnique < 4) { skipped++; return; }
    { uint64_t b[4] = {v[4], v[7], v[6], v[5]}; if (allSame(0, 1, 2, 3)) { tryPyramid(b, v[0], numUnique, out, skipped); return; } }
    { uint64_t b[4] = {v[0], v[1], v[2], v[3]}; if (allSame(4, 5, 6, 7)) { tryPyramid(b, v[4], numUnique, out, skipped); return; } }
    { uint64_t b[4] = {v[2], v[6], v[7], v[3]}; if (allSame(0, 1, 4, 5)) { tryPyramid(b, v[0], numUnique, out, skipped); return; } }
    { uint64_t b[4] = {v[0], v[4], v[5], v[1]}; if (allSame(2, 3, 6, 7)) { tryPyramid(b, v[2], numUnique, out, skipped); return; } }
    { uint64_t b[4] = {v[1], v[5], v[6], v[2]}; if (allSame(0, 3, 4, 7)) { tryPyramid(b, v[0], numUnique, out, skipped); return; } }
    { uint64_t b[4] = {v[0], v[3], v[7], v[4]}; if (allSame(1, 2, 5, 6)) { tryPyramid(b, v[1], numUnique, out, skipped); return; } }
    if (same(0, 1) && same(4, 5)) { wedge(v, 3, 2, 0, 7, 6, 4, out); return; }
    if (same(0, 4) && same(1, 5)) { wedge(v, 2, 6, 5, 3, 7, 4, out); return; }
    if (same(3, 7) && same(2, 6)) { wedge(v, 5, 1, 2, 4, 0, 3, out); return; }
    if (same(2, 3) && same(6, 7)) { wedge(v, 1, 0, 3, 5, 4, 7, out); return; }
    if (same(4, 7) && same(5, 6)) { wedge(v, 3, 0, 4, 2, 1, 6, out); return; }
    if (same(4, 5) && same(6, 7)) { wedge(v, 0, 1, 4, 3, 2, 7, out); return; }
    if (same(0, 1) && same(3, 2)) { wedge(v, 5, 4, 0, 6, 7, 3, out); return; }
    if (same(0, 3) && same(1, 2)) { wedge(v, 4, 7, 3, 5, 6, 2, out); return; }
    if (same(0, 3) && same(4, 7)) { wedge(v, 5, 6, 7, 1, 2, 3, out); return; }
    if (same(0, 4) && same(3, 7)) { wedge(v, 1, 5, 4, 2, 6, 7, out); return; }
    if (same(1, 2) && same(5, 6)) { wedge(v, 7, 4, 5, 3, 0, 1, out); return; }
    if (same(1, 5) && same(2, 6)) { wedge(v, 4, 0, 1, 7, 3, 2, out); return; }
    hex(v, out);
  }

  void buildElements()
  {
    const int nt = numThreadsOf(&P);
    // process leaves in fixed chunks; concatenate chunk outputs in order
    struct Chunk { int L; int64_t w0, w1; };
    std::vector<Chunk> chunks;
    for (int L = 0; L <= Lroot; ++L) {
      const int64_t nw = (int64_t)lv[L].leaf.w.size();
      for (int64_t w = 0; w < nw; w += 1024) chunks.push_back({L, w, std::min(nw, w + 1024)});
    }
    std::vector<std::vector<Elem>> outs(chunks.size() * 4);
    std::vector<uint64_t> skippedPer(chunks.size(), 0);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t ch = 0; ch < (int64_t)chunks.size(); ++ch) {
      const Chunk &C = chunks[ch];
      const Level &l = lv[C.L];
      for (int64_t wi = C.w0; wi < C.w1; ++wi) {
        uint64_t word = l.leaf.w[wi];
        while (word) {
          const int b = __builtin_ctzll(word);
          word &= word - 1;
          const uint64_t c = (uint64_t)wi * 64 + b;
          const int64_t i = c % l.n[0], j = (c / l.n[0]) % l.n[1], k = c / (l.n[0] * l.n[1]);
          doCell(C.L, i, j, k, &outs[ch * 4], skippedPer[ch]);
        }
      }
    }
    std::vector<Elem> elems;
    uint64_t counts[4] = {0, 0, 0, 0};
    for (int t = 0; t < 4; ++t)
      for (size_t ch = 0; ch < chunks.size(); ++ch) {
        const auto &o = outs[ch * 4 + t];
        elems.insert(elems.end(), o.begin(), o.end());
        counts[t] += o.size();
      }
    for (auto s : skippedPer) R.stats.numSkippedDegenerate += s;
    R.stats.numTets = counts[0]; R.stats.numPyramids = counts[1];
    R.stats.numWedges = counts[2]; R.stats.numHexes = counts[3];
    // vertex compaction: used leaves in ascending leaf id
    std::vector<uint32_t> used;
    used.reserve(elems.size() * 6);
    static const int nv[4] = {4, 5, 6, 8};
    for (const Elem &e : elems)
      for (int i = 0; i < nv[e.type]; ++i) used.push_back(e.v[i]);
    std::sort(used.begin(), used.end());
    used.erase(std::unique(used.begin(), used.end()), used.end());
    R.vertices.resize(used.size());
    const std::vector<int32_t> &cells = R.amrCells;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)used.size(); ++i) {
      const uint32_t id = used[i];
      const int L = cells[(uint64_t)id * 4 + 3];
      const float h = 0.5f * (float)(1 << L);
      exa_vec4f v;
      v.x = (float)cells[(uint64_t)id * 4 + 0] + h;
      v.y = (float)cells[(uint64_t)id * 4 + 1] + h;
      v.z = (float)cells[(uint64_t)id * 4 + 2] + h;
      v.w = value[id];
      R.vertices[i] = v;
    }
    R.indices.assign(elems.size() * 8, -1);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t e = 0; e < (int64_t)elems.size(); ++e) {
      const Elem &E = elems[e];
      for (int i = 0; i < nv[E.type]; ++i)
        R.indices[e * 8 + i] = (int32_t)(std::lower_bound(used.begin(), used.end(), E.v[i]) - used.begin());
    }
    R.stats.numVertices = used.size();
  }

  // ---- makeGrids.cpp:57-209: perfect cubes -> 8^3 bricks ----
  // A perfect cube of level L has its min corner at (i,j,k) when the 2x2x2
  // block of level-L cells there are all leaves.  Cubes are grouped by
  // macrocell (i/8, j/8, k/8) (makeGrids.cpp:79-93); the brick spans the
  // bounding box of its cubes' cells; vertices no cube writes stay NaN.
  void buildGridlets()
  {
    const int nt = numThreadsOf(&P);
    const int MCW = 8;  // makeGrids.cpp:46
    for (int L = 0; L <= Lroot; ++L) {
      const Level &l = lv[L];
      const std::vector<uint64_t> &W = l.leaf.w;
      // leaf bits of cells x0..x0+8 of row (j,k)
      auto rowBits = [&](int64_t x0, int64_t j, int64_t k) -> uint32_t {
        if (j >= l.n[1] || k >= l.n[2] || x0 >= l.n[0]) return 0;
        const uint64_t b = l.lin(x0, j, k);
        uint64_t w0 = W[b >> 6] >> (b & 63);
        if ((b & 63) > 55 && (b >> 6) + 1 < W.size()) w0 |= W[(b >> 6) + 1] << (64 - (b & 63));
        uint32_t m = (uint32_t)(w0 & 0x1ffu);
        const int64_t valid = l.n[0] - x0;
        if (valid < 9) m &= (1u << valid) - 1u;
        return m;
      };
      const int64_t m[3] = {(l.n[0] + MCW - 1) / MCW, (l.n[1] + MCW - 1) / MCW, (l.n[2] + MCW - 1) / MCW};
      const uint64_t nmc = (uint64_t)m[0] * m[1] * m[2];
      std::vector<uint32_t> cnt(nmc, 0);
      std::vector<int32_t> box(nmc * 6);
      // cube masks of one macrocell: bit t of mask[kk*8+jj] = cube at (x0+t, y0+jj, z0+kk)
      auto cubeMasks = [&](uint64_t mc, uint8_t *mask) {
        const int64_t mx = mc % m[0], my = (mc / m[0]) % m[1], mz = mc / (m[0] * m[1]);
        const int64_t x0 = mx * MCW, y0 = my * MCW, z0 = mz * MCW;
        uint32_t rows[9][9];
        for (int kk = 0; kk < 9; ++kk)
          for (int jj = 0; jj < 9; ++jj) rows[kk][jj] = rowBits(x0, y0 + jj, z0 + kk);
        for (int kk = 0; kk < 8; ++kk)
          for (int jj = 0; jj < 8; ++jj) {
            const uint32_t a = rows[kk][jj] & rows[kk][jj + 1] & rows[kk + 1][jj] & rows[kk + 1][jj + 1];
            mask[kk * 8 + jj] = (uint8_t)(a & (a >> 1) & 0xffu);
          }
      };
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
      for (int64_t mc = 0; mc < (int64_t)nmc; ++mc) {
        uint8_t mask[64];
        cubeMasks((uint64_t)mc, mask);
        const int64_t mx = mc % m[0], my = (mc / m[0]) % m[1], mz = mc / (m[0] * m[1]);
        int32_t lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
        uint32_t c = 0;
        for (int kk = 0; kk < 8; ++kk)
          for (int jj = 0; jj < 8; ++jj) {
            const uint32_t bm = mask[kk * 8 + jj];
            if (!bm) continue;
            c += (uint32_t)__builtin_popcount(bm);
            const int32_t i0 = (int32_t)(mx * MCW) + __builtin_ctz(bm);
            const int32_t i1 = (int32_t)(mx * MCW) + 31 - __builtin_clz(bm);
            const int32_t j = (int32_t)(my * MCW + jj), k = (int32_t)(mz * MCW + kk);
            lo[0] = std::min(lo[0], i0); hi[0] = std::max(hi[0], i1 + 1);
            lo[1] = std::min(lo[1], j); hi[1] = std::max(hi[1], j + 1);
            lo[2] = std::min(lo[2], k); hi[2] = std::max(hi[2], k + 1);
          }
        cnt[mc] = c;
        for (int a = 0; a < 3; ++a) { box[mc * 6 + a] = lo[a]; box[mc * 6 + 3 + a] = hi[a]; }
      }
      // bricks in ascending macrocell order
      std::vector<int64_t> brickOf(nmc, -1);
      uint64_t numCubes = 0;
      for (uint64_t mc = 0; mc < nmc; ++mc) {
        if (!cnt[mc]) continue;
        numCubes += cnt[mc];
        exa_gridlet g;
        g.lower = {box[mc * 6], box[mc * 6 + 1], box[mc * 6 + 2]};
        g.level = L;
        g.dims = {box[mc * 6 + 3] - box[mc * 6], box[mc * 6 + 4] - box[mc * 6 + 1], box[mc * 6 + 5] - box[mc * 6 + 2]};
        const uint64_t ns = (uint64_t)(g.dims.x + 1) * (g.dims.y + 1) * (g.dims.z + 1);
        if (R.gridletScalars.size() + ns > 0xffffffffull) throw std::runtime_error("gridlet scalar offset overflow");
        g.begin = (uint32_t)R.gridletScalars.size();
        brickOf[mc] = (int64_t)R.gridlets.size();
        R.gridlets.push_back(g);
        R.gridletScalars.resize(R.gridletScalars.size() + ns, NAN);
      }
      R.stats.numPerfectCubes += numCubes;
      // corner values (Brick::write, makeGrids.cpp:114-168)
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
      for (int64_t mc = 0; mc < (int64_t)nmc; ++mc) {
        if (!cnt[mc]) continue;
        uint8_t mask[64];
        cubeMasks((uint64_t)mc, mask);
        const int64_t mx = mc % m[0], my = (mc / m[0]) % m[1], mz = mc / (m[0] * m[1]);
        const exa_gridlet &g = R.gridlets[brickOf[mc]];
        const int64_t nx = g.dims.x + 1, ny = g.dims.y + 1;
        for (int kk = 0; kk < 8; ++kk)
          for (int jj = 0; jj < 8; ++jj) {
            uint32_t bm = mask[kk * 8 + jj];
            while (bm) {
              const int t = __builtin_ctz(bm);
              bm &= bm - 1;
              const int64_t i = mx * MCW + t, j = my * MCW + jj, k = mz * MCW + kk;
              for (int d = 0; d < 8; ++d) {
                const int64_t ix = d & 1, iy = (d >> 1) & 1, iz = d >> 2;
                const uint64_t cc = l.lin(i + ix, j + iy, k + iz);
                const uint64_t id = l.leafOffset + l.leaf.rankOf(cc);
                const int64_t lx = i + ix - g.lower.x, ly = j + iy - g.lower.y, lz = k + iz - g.lower.z;
                R.gridletScalars[g.begin + (uint64_t)((lz * ny + ly) * nx + lx)] = value[id];
              }
            }
          }
      }
    }
    uint64_t empty = 0;
    for (float v : R.gridletScalars) if (std::isnan(v)) empty++;
    R.stats.numGridlets = R.gridlets.size();
    R.stats.numGridletScalars = R.gridletScalars.size();
    R.stats.numEmptyGridletScalars = empty;
  }
};

} // namespace

extern "C" {

void exa_gen_params_default(exa_gen_params *p)
{
  std::memset(p, 0, sizeof(*p));
  p->numLevels = 3;
  p->rootDims[0] = p->rootDims[1] = p->rootDims[2] = 32;
  p->fieldKind = EXA_FIELD_GAUSSIANS;
  p->numGaussians = 32;
  p->seed = 1234;
  p->refineThreshold = 0.5f;
  p->noiseAmplitude = 0.1f;
  p->noiseOctaves = 4;
  p->cloudEmptyFraction = 0.7f;
  p->balance = 1;
  p->numThreads = 0;
}

int exa_gen_run(const exa_gen_params *p, exa_gen_result **out)
{
  try {
    if (!out) throw std::runtime_error("null argument");
    exagen::checkParams(p);
    auto t0 = std::chrono::steady_clock::now();
    exa_gen_result *r = new exa_gen_result();
    r->params = *p;
    std::memset(&r->stats, 0, sizeof(r->stats));
    Builder B(*p, *r);
    auto stage = [&](int k, auto &&fn) {
      const auto a = std::chrono::steady_clock::now();
      fn();
      r->stats.stageSeconds[k] = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
    };
    stage(0, [&] { B.setupField(); });
    stage(1, [&] { B.buildGaussTables(); });
    stage(2, [&] { B.buildTree(); });
    if (r->stats.numAmrCells >= 0x7fffffffull) throw std::runtime_error("too many AMR cells for 32-bit ids");
    stage(3, [&] { B.computeValues(); });
    stage(4, [&] { B.buildElements(); });
    stage(5, [&] { B.buildGridlets(); });
    r->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = r;
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

void exa_gen_free(exa_gen_result *r) { delete r; }

void exa_gen_get_stats(const exa_gen_result *r, exa_gen_stats *s) { *s = r->stats; }

const exa_vec4f *exa_gen_vertices(const exa_gen_result *r, uint64_t *n)
{
  *n = r->vertices.size();
  return r->vertices.data();
}
const int32_t *exa_gen_indices(const exa_gen_result *r, uint64_t *n)
{
  *n = r->indices.size() / 8;
  return r->indices.data();
}
const exa_gridlet *exa_gen_gridlets(const exa_gen_result *r, uint64_t *n)
{
  *n = r->gridlets.size();
  return r->gridlets.data();
}
const float *exa_gen_gridlet_scalars(const exa_gen_result *r, uint64_t *n)
{
  *n = r->gridletScalars.size();
  return r->gridletScalars.data();
}
const int32_t *exa_gen_amr_cells(const exa_gen_result *r, uint64_t *n)
{
  *n = r->amrCells.size() / 4;
  return r->amrCells.data();
}
const float *exa_gen_amr_scalars(const exa_gen_result *r, uint64_t *n)
{
  *n = r->amrScalars.size();
  return r->amrScalars.data();
}

void exa_gen_eval_field(const exa_gen_result *r, const exa_vec3f *pos, uint64_t n, float *out)
{
  const Field &F = r->field;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    out[i] = (float)F.evalUnit(pos[i].x / F.extent[0], pos[i].y / F.extent[1], pos[i].z / F.extent[2]);
}

const char *exa_gen_last_error(void) { return g_err.c_str(); }

} // extern "C"

// Once-per-mesh host preparation: validation, renumbering for the DIC order,
// scheduling parts for the triangular sweeps, and the cell-to-face CSR in the
// storage order used on the device.
//
// DIC is defined by the cell numbering (OpenFOAM DICPreconditioner: the lower
// triangle is the set of faces seen from their higher-numbered cell).  Three
// numberings are offered (s4g_renumber): the caller's, reverse Cuthill-McKee,
// and a tiled part-major numbering from recursive coordinate bisection.  The
// device stores rows in a topological order of that numbering's
// lower-triangular DAG -- contiguous parts, and inside each part rows sorted
// by their in-part level -- which keeps every face's lower/upper role, so the
// incomplete-Cholesky factor and both sweeps equal those of the chosen
// numbering exactly (up to the summation order of floating point).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>

#include "s4g_internal.hpp"

namespace s4g {
namespace {

struct Adj {
  std::vector<int> ptr, cell, face;
};

Adj buildAdjacency(int nC, int nI, const int* own, const int* nei) {
  Adj a;
  a.ptr.assign(nC + 1, 0);
  for (int f = 0; f < nI; ++f) { a.ptr[own[f] + 1]++; a.ptr[nei[f] + 1]++; }
  for (int c = 0; c < nC; ++c) a.ptr[c + 1] += a.ptr[c];
  a.cell.resize(2 * (size_t)nI);
  a.face.resize(2 * (size_t)nI);
  std::vector<int> fill(a.ptr.begin(), a.ptr.end() - 1);
  for (int f = 0; f < nI; ++f) {
    a.cell[fill[own[f]]] = nei[f]; a.face[fill[own[f]]++] = f;
    a.cell[fill[nei[f]]] = own[f]; a.face[fill[nei[f]]++] = f;
  }
  return a;
}

// Breadth-first order of the cells in `set` (a subgraph given by mask==tag)
// from `start`; returns visit order and the last level's first node.
std::vector<int> bfs(const Adj& a, const std::vector<int>& mask, int tag, int start,
                     std::vector<int>& level, bool sortByDegree) {
  std::vector<int> order;
  std::queue<int> q;
  q.push(start);
  level[start] = 0;
  std::vector<int> nb;
  while (!q.empty()) {
    int c = q.front(); q.pop();
    order.push_back(c);
    nb.clear();
    for (int e = a.ptr[c]; e < a.ptr[c + 1]; ++e) {
      int o = a.cell[e];
      if (mask[o] != tag || level[o] >= 0) continue;
      level[o] = level[c] + 1;
      nb.push_back(o);
    }
    if (sortByDegree)
      std::stable_sort(nb.begin(), nb.end(), [&](int x, int y) {
        return (a.ptr[x + 1] - a.ptr[x]) < (a.ptr[y + 1] - a.ptr[y]);
      });
    for (int o : nb) q.push(o);
  }
  return order;
}

// Pseudo-peripheral node of the subgraph containing `seed` (two BFS sweeps).
int peripheral(const Adj& a, const std::vector<int>& mask, int tag, int seed,
               std::vector<int>& level) {
  int node = seed;
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int> ord = bfs(a, mask, tag, node, level, false);
    int far = ord.back();
    int best = far;
    int maxL = level[far];
    for (int c : ord)
      if (level[c] == maxL &&
          (a.ptr[c + 1] - a.ptr[c]) < (a.ptr[best + 1] - a.ptr[best]))
        best = c;
    for (int c : ord) level[c] = -1;
    node = best;
  }
  return node;
}

// Ordering of a (possibly disconnected) subgraph: BFS/Cuthill-McKee per
// component from pseudo-peripheral nodes.
std::vector<int> orderSubgraph(const Adj& a, const std::vector<int>& cells,
                               std::vector<int>& mask, int tag, std::vector<int>& level,
                               bool cuthillMcKee) {
  std::vector<int> out;
  out.reserve(cells.size());
  for (int c : cells) { mask[c] = tag; level[c] = -1; }
  std::vector<int> byDeg(cells);
  std::stable_sort(byDeg.begin(), byDeg.end(), [&](int x, int y) {
    return (a.ptr[x + 1] - a.ptr[x]) < (a.ptr[y + 1] - a.ptr[y]);
  });
  for (int seed : byDeg) {
    if (level[seed] >= 0) continue;
    int st = peripheral(a, mask, tag, seed, level);
    std::vector<int> ord = bfs(a, mask, tag, st, level, cuthillMcKee);
    out.insert(out.end(), ord.begin(), ord.end());
  }
  for (int c : cells) mask[c] = -1;
  return out;
}

void rcbSplit(const double* C, std::vector<int>& cells, size_t lo, size_t hi,
              int partSize, std::vector<std::pair<size_t, size_t>>& parts) {
  if (hi - lo <= (size_t)partSize) { parts.push_back({lo, hi}); return; }
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (size_t i = lo; i < hi; ++i)
    for (int k = 0; k < 3; ++k) {
      double v = C[3 * (size_t)cells[i] + k];
      mn[k] = std::min(mn[k], v); mx[k] = std::max(mx[k], v);
    }
  int ax = 0;
  for (int k = 1; k < 3; ++k) if (mx[k] - mn[k] > mx[ax] - mn[ax] + 1e-12 * (mx[ax] - mn[ax])) ax = k;
  size_t mid = lo + (hi - lo) / 2;
  std::nth_element(cells.begin() + lo, cells.begin() + mid, cells.begin() + hi,
                   [&](int x, int y) {
                     double vx = C[3 * (size_t)x + ax], vy = C[3 * (size_t)y + ax];
                     return vx != vy ? vx < vy : x < y;
                   });
  rcbSplit(C, cells, lo, mid, partSize, parts);
  rcbSplit(C, cells, mid, hi, partSize, parts);
}

}  // namespace

s4g_status prepareMesh(const s4g_mesh_desc* d, const s4g_mesh_opts* o, HostPrep& hp,
                       std::string& err) {
  const int nC = d->n_cells, nF = d->n_faces, nI = d->n_internal_faces;
  const int nB = nF - nI;
  if (nC <= 0 || nI < 0 || nB < 0 || !d->owner || (nI > 0 && !d->neighbour) || !d->C ||
      !d->V || !d->Cf || !d->Sf || d->n_patches < 0 ||
      (d->n_patches > 0 && (!d->patch_start || !d->patch_size))) {
    err = "missing or inconsistent mesh arrays";
    return S4G_BAD_ARG;
  }
  for (int f = 0; f < nF; ++f)
    if (d->owner[f] < 0 || d->owner[f] >= nC) { err = "owner out of range"; return S4G_BAD_ARG; }
  for (int f = 0; f < nI; ++f)
    if (d->neighbour[f] < 0 || d->neighbour[f] >= nC || d->neighbour[f] == d->owner[f]) {
      err = "neighbour out of range or equal to owner";
      return S4G_BAD_ARG;
    }
  {
    long long covered = 0;
    int expect = nI;
    for (int p = 0; p < d->n_patches; ++p) {
      if (d->patch_start[p] != expect || d->patch_size[p] < 0) {
        err = "patches must cover the boundary faces contiguously in order";
        return S4G_BAD_ARG;
      }
      expect += d->patch_size[p];
      covered += d->patch_size[p];
    }
    if (covered != nB) { err = "patch sizes do not add up to the boundary faces"; return S4G_BAD_ARG; }
  }
  for (long i = 0; i < 3L * nC; ++i)
    if (!std::isfinite(d->C[i])) { err = "non-finite cell centre"; return S4G_BAD_ARG; }
  for (int c = 0; c < nC; ++c)
    if (!(d->V[c] > 0)) { err = "non-positive cell volume"; return S4G_BAD_ARG; }
  for (long i = 0; i < 3L * nF; ++i)
    if (!std::isfinite(d->Sf[i]) || !std::isfinite(d->Cf[i])) {
      err = "non-finite face geometry";
      return S4G_BAD_ARG;
    }

  if (o && (o->empty_direction < 0 || o->empty_direction > 3)) {
    err = "empty_direction must be 0 (3-D) or 1, 2, 3 (x, y, z)";
    return S4G_BAD_ARG;
  }
  const int renumber = o ? (int)o->renumber : (int)S4G_RENUMBER_TILED;
  int partSize = (o && o->part_size > 0) ? o->part_size : 512;
  partSize = std::max(32, std::min(partSize, 1 << 16));
  const bool subdomains = o && o->dic_subdomains;
  // the caller's decomposition (decomposePar's cellDecomposition): ids
  // 0..n-1, none empty; each subdomain's DIC runs in the caller's order
  const int* callerParts = o ? o->part_of_cell : nullptr;
  int nCallerParts = 0;
  if (callerParts) {
    if (renumber != S4G_RENUMBER_NONE || !subdomains) {
      err = "part_of_cell needs renumber = S4G_RENUMBER_NONE and dic_subdomains = 1";
      return S4G_BAD_ARG;
    }
    for (int c = 0; c < nC; ++c) {
      if (callerParts[c] < 0 || callerParts[c] >= nC) { err = "part_of_cell id out of range"; return S4G_BAD_ARG; }
      nCallerParts = std::max(nCallerParts, callerParts[c] + 1);
    }
    std::vector<int> cnt(nCallerParts, 0);
    for (int c = 0; c < nC; ++c) cnt[callerParts[c]]++;
    for (int p = 0; p < nCallerParts; ++p)
      if (cnt[p] == 0) { err = "part_of_cell ids must be 0..n-1 with every id used"; return S4G_BAD_ARG; }
  }

  hp.nC = nC; hp.nI = nI; hp.nB = nB;
  Adj adj = buildAdjacency(nC, nI, d->owner, d->neighbour);
  std::vector<int> mask(nC, -1), level(nC, -1);

  // ---- 1. solver (DIC) order: solver rank -> caller cell
  std::vector<int> order;
  std::vector<std::pair<size_t, size_t>> tiles;  // TILED parts in `order`
  if (renumber == S4G_RENUMBER_NONE) {
    order.resize(nC);
    std::iota(order.begin(), order.end(), 0);
  } else if (renumber == S4G_RENUMBER_RCM) {
    std::vector<int> all(nC);
    std::iota(all.begin(), all.end(), 0);
    order = orderSubgraph(adj, all, mask, 0, level, true);
    std::reverse(order.begin(), order.end());
  } else if (renumber == S4G_RENUMBER_TILED) {
    std::vector<int> cells(nC);
    std::iota(cells.begin(), cells.end(), 0);
    std::vector<std::pair<size_t, size_t>> leaves;
    rcbSplit(d->C, cells, 0, (size_t)nC, partSize, leaves);
    const int nL = (int)leaves.size();
    std::vector<int> partOf(nC);
    for (int p = 0; p < nL; ++p)
      for (size_t i = leaves[p].first; i < leaves[p].second; ++i) partOf[cells[i]] = p;
    // part graph
    Adj pg;
    {
      std::vector<std::vector<int>> nbs(nL);
      for (int f = 0; f < nI; ++f) {
        int a = partOf[d->owner[f]], b = partOf[d->neighbour[f]];
        if (a != b) { nbs[a].push_back(b); nbs[b].push_back(a); }
      }
      pg.ptr.assign(nL + 1, 0);
      for (int p = 0; p < nL; ++p) {
        std::sort(nbs[p].begin(), nbs[p].end());
        nbs[p].erase(std::unique(nbs[p].begin(), nbs[p].end()), nbs[p].end());
        pg.ptr[p + 1] = pg.ptr[p] + (int)nbs[p].size();
      }
      for (int p = 0; p < nL; ++p) pg.cell.insert(pg.cell.end(), nbs[p].begin(), nbs[p].end());
    }
    std::vector<int> pmask(nL, -1), plevel(nL, -1), allp(nL);
    std::iota(allp.begin(), allp.end(), 0);
    std::vector<int> porder = orderSubgraph(pg, allp, pmask, 0, plevel, false);
    order.reserve(nC);
    for (int p : porder) {
      std::vector<int> pc(cells.begin() + leaves[p].first, cells.begin() + leaves[p].second);
      std::sort(pc.begin(), pc.end());
      std::vector<int> loc = orderSubgraph(adj, pc, mask, 1, level, false);
      size_t st = order.size();
      order.insert(order.end(), loc.begin(), loc.end());
      tiles.push_back({st, order.size()});
    }
  } else {
    err = "unknown renumber option";
    return S4G_BAD_ARG;
  }
  std::vector<int> rank(nC);
  for (int i = 0; i < nC; ++i) rank[order[i]] = i;

  // ---- 2. global DAG levels in the solver order
  std::vector<int> glev(nC, 0);
  int gmax = 0;
  for (int i = 0; i < nC; ++i) {
    int c = order[i], l = 0;
    for (int e = adj.ptr[c]; e < adj.ptr[c + 1]; ++e) {
      int o2 = adj.cell[e];
      if (rank[o2] < i) l = std::max(l, glev[o2] + 1);
    }
    glev[c] = l;
    gmax = std::max(gmax, l);
  }
  hp.globalLevels = gmax + 1;

  // ---- 3. topological storage order split into parts
  std::vector<int> topo;  // storage candidates (caller cells) before in-part sorting
  std::vector<std::pair<size_t, size_t>> parts;
  if (renumber == S4G_RENUMBER_TILED) {
    topo = order;
    parts = tiles;
  } else if (callerParts) {
    // cells grouped by the caller's subdomain, each in solver order
    std::vector<size_t> at(nCallerParts + 1, 0);
    for (int c = 0; c < nC; ++c) at[callerParts[c] + 1]++;
    for (int p = 0; p < nCallerParts; ++p) at[p + 1] += at[p];
    for (int p = 0; p < nCallerParts; ++p) parts.push_back({at[p], at[p + 1]});
    topo.resize(nC);
    for (int i = 0; i < nC; ++i) {
      const int c = order[i];
      topo[at[callerParts[c]]++] = c;
    }
  } else {
    topo = order;
    std::stable_sort(topo.begin(), topo.end(), [&](int x, int y) { return glev[x] < glev[y]; });
    for (size_t s = 0; s < (size_t)nC; s += partSize)
      parts.push_back({s, std::min((size_t)nC, s + partSize)});
  }
  hp.nParts = (int)parts.size();
  std::vector<int> partOfCell(nC);
  for (int p = 0; p < hp.nParts; ++p)
    for (size_t i = parts[p].first; i < parts[p].second; ++i) partOfCell[topo[i]] = p;

  // in-part levels (in solver order), then sort each part by (level, rank)
  std::vector<int> llev(nC, 0);
  hp.s2c.resize(nC);
  hp.partStart.assign(hp.nParts + 1, 0);
  hp.lvlOff.assign(hp.nParts + 1, 0);
  hp.lvlStart.clear();
  hp.maxLocalLevels = 0;
  for (int p = 0; p < hp.nParts; ++p) {
    std::vector<int> pc(topo.begin() + parts[p].first, topo.begin() + parts[p].second);
    std::sort(pc.begin(), pc.end(), [&](int x, int y) { return rank[x] < rank[y]; });
    int nl = 0;
    for (int c : pc) {
      int l = 0;
      for (int e = adj.ptr[c]; e < adj.ptr[c + 1]; ++e) {
        int o2 = adj.cell[e];
        if (rank[o2] < rank[c] && partOfCell[o2] == p) l = std::max(l, llev[o2] + 1);
      }
      llev[c] = l;
      nl = std::max(nl, l + 1);
    }
    std::stable_sort(pc.begin(), pc.end(), [&](int x, int y) { return llev[x] < llev[y]; });
    int st = (int)parts[p].first;
    hp.partStart[p] = st;
    hp.lvlOff[p] = (int)hp.lvlStart.size();
    int prev = -1;
    for (size_t i = 0; i < pc.size(); ++i) {
      hp.s2c[st + i] = pc[i];
      while (prev < llev[pc[i]]) { hp.lvlStart.push_back(st + (int)i); ++prev; }
    }
    hp.maxLocalLevels = std::max(hp.maxLocalLevels, nl);
  }
  hp.partStart[hp.nParts] = nC;
  hp.lvlStart.push_back(nC);  // sentinel; each part's last level ends at the next part's first
  hp.lvlOff[hp.nParts] = (int)hp.lvlStart.size() - 1;
  hp.c2s.resize(nC);
  for (int s = 0; s < nC; ++s) hp.c2s[hp.s2c[s]] = s;
  hp.solverRank.resize(nC);
  for (int s = 0; s < nC; ++s) hp.solverRank[s] = rank[hp.s2c[s]];

  // ---- 4. internal faces in storage orientation, sorted by (owner, neighbour)
  // (a counting sort by the storage owner, then each owner's few faces by
  // neighbour, in face order among equal pairs)
  std::vector<int> fidxOrder(nI);
  auto so = [&](int f) { return std::min(hp.c2s[d->owner[f]], hp.c2s[d->neighbour[f]]); };
  auto sn = [&](int f) { return std::max(hp.c2s[d->owner[f]], hp.c2s[d->neighbour[f]]); };
  {
    std::vector<int> start(nC + 1, 0);
    for (int f = 0; f < nI; ++f) ++start[so(f) + 1];
    for (int s = 0; s < nC; ++s) start[s + 1] += start[s];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int f = 0; f < nI; ++f) fidxOrder[fill[so(f)]++] = f;
    for (int s = 0; s < nC; ++s)
      for (int a = start[s] + 1; a < start[s + 1]; ++a) {
        const int f = fidxOrder[a], key = sn(f);
        int b = a;
        for (; b > start[s] && sn(fidxOrder[b - 1]) > key; --b) fidxOrder[b] = fidxOrder[b - 1];
        fidxOrder[b] = f;
      }
  }
  hp.fown.resize(nI); hp.fnei.resize(nI); hp.fcaller.resize(nI); hp.fflip.resize(nI);
  std::vector<int> fnew(nI);
  for (int k = 0; k < nI; ++k) {
    int f = fidxOrder[k];
    hp.fown[k] = so(f); hp.fnei[k] = sn(f); hp.fcaller[k] = f;
    hp.fflip[k] = hp.c2s[d->owner[f]] > hp.c2s[d->neighbour[f]];
    fnew[f] = k;
  }

  // ---- 5. CSR rows in storage order: lower entries (by solver rank), then upper
  hp.rowptr.assign(nC + 1, 0);
  for (int s = 0; s < nC; ++s) {
    int c = hp.s2c[s];
    hp.rowptr[s + 1] = hp.rowptr[s] + (adj.ptr[c + 1] - adj.ptr[c]);
  }
  hp.col.resize(2 * (size_t)nI);
  hp.fidx.resize(2 * (size_t)nI);
  {
    std::vector<std::pair<int, int>> ent;
    for (int s = 0; s < nC; ++s) {
      int c = hp.s2c[s];
      ent.clear();
      for (int e = adj.ptr[c]; e < adj.ptr[c + 1]; ++e) ent.push_back({adj.cell[e], adj.face[e]});
      // a row's few neighbours by solver rank (distinct): insertion sort
      for (size_t a = 1; a < ent.size(); ++a) {
        const std::pair<int, int> v = ent[a];
        size_t b = a;
        for (; b > 0 && rank[ent[b - 1].first] > rank[v.first]; --b) ent[b] = ent[b - 1];
        ent[b] = v;
      }
      int k = hp.rowptr[s];
      for (auto& pr : ent) {
        int ns = hp.c2s[pr.first];
        int fk = fnew[pr.second];
        hp.col[k] = ns;
        hp.fidx[k] = (hp.fown[fk] == s) ? fk : ~fk;
        ++k;
      }
    }
  }

  // ---- 6. boundary faces sorted by storage cell
  {
    std::vector<int> bf(nB);
    std::iota(bf.begin(), bf.end(), 0);
    std::stable_sort(bf.begin(), bf.end(), [&](int a, int b) {
      return hp.c2s[d->owner[nI + a]] < hp.c2s[d->owner[nI + b]];
    });
    std::vector<int> patchOf(nB);
    for (int p = 0; p < d->n_patches; ++p)
      for (int i = 0; i < d->patch_size[p]; ++i) patchOf[d->patch_start[p] + i - nI] = p;
    hp.bcell.resize(nB); hp.bpatch.resize(nB); hp.bcaller.resize(nB);
    hp.browptr.assign(nC + 1, 0);
    for (int k = 0; k < nB; ++k) {
      int b = bf[k];
      hp.bcell[k] = hp.c2s[d->owner[nI + b]];
      hp.bpatch[k] = patchOf[b];
      hp.bcaller[k] = b;
      hp.browptr[hp.bcell[k] + 1]++;
    }
    for (int s = 0; s < nC; ++s) hp.browptr[s + 1] += hp.browptr[s];
  }

  // ---- 7. part dependencies
  hp.upPtr.assign(hp.nParts + 1, 0);
  hp.dnPtr.assign(hp.nParts + 1, 0);
  hp.upIdx.clear(); hp.dnIdx.clear();
  std::vector<int> partOfRow(nC);
  for (int p = 0; p < hp.nParts; ++p)
    for (int s = hp.partStart[p]; s < hp.partStart[p + 1]; ++s) partOfRow[s] = p;
  std::vector<std::vector<int>> dn(hp.nParts);
  std::vector<int> depth(hp.nParts, 1);
  hp.partDepth = hp.nParts > 0 ? 1 : 0;
  for (int p = 0; p < hp.nParts; ++p) {
    std::vector<int> ups;
    if (!subdomains) {
      for (int s = hp.partStart[p]; s < hp.partStart[p + 1]; ++s)
        for (int k = hp.rowptr[s]; k < hp.rowptr[s + 1]; ++k) {
          int q = partOfRow[hp.col[k]];
          if (hp.col[k] < s && q != p) ups.push_back(q);
        }
      std::sort(ups.begin(), ups.end());
      ups.erase(std::unique(ups.begin(), ups.end()), ups.end());
    }
    for (int q : ups) {
      if (q >= p) { err = "internal error: part order is not topological"; return S4G_BAD_ARG; }
      dn[q].push_back(p);
      depth[p] = std::max(depth[p], depth[q] + 1);
    }
    hp.partDepth = std::max(hp.partDepth, depth[p]);
    hp.upIdx.insert(hp.upIdx.end(), ups.begin(), ups.end());
    hp.upPtr[p + 1] = (int)hp.upIdx.size();
  }
  for (int p = 0; p < hp.nParts; ++p) {
    hp.dnIdx.insert(hp.dnIdx.end(), dn[p].begin(), dn[p].end());
    hp.dnPtr[p + 1] = (int)hp.dnIdx.size();
  }

  // ---- 8. shared-memory staging tables of the sweeps
  hp.lowCnt.assign(nC, 0);
  for (int s = 0; s < nC; ++s)
    for (int k = hp.rowptr[s]; k < hp.rowptr[s + 1]; ++k)
      if (hp.col[k] < s) hp.lowCnt[s]++;
  hp.maxRows = 0; hp.maxHalo = 0; hp.maxEntries = 0;
  for (int p = 0; p < hp.nParts; ++p) {
    hp.maxRows = std::max(hp.maxRows, hp.partStart[p + 1] - hp.partStart[p]);
    hp.maxEntries = std::max(hp.maxEntries, hp.rowptr[hp.partStart[p + 1]] - hp.rowptr[hp.partStart[p]]);
  }
  hp.haloFPtr.assign(hp.nParts + 1, 0);
  hp.haloBPtr.assign(hp.nParts + 1, 0);
  hp.haloFIdx.clear(); hp.haloBIdx.clear();
  hp.slot.assign(hp.col.size(), 0);
  {
    std::vector<int> hf, hb;
    for (int p = 0; p < hp.nParts; ++p) {
      const int lo = hp.partStart[p], hi = hp.partStart[p + 1];
      hf.clear(); hb.clear();
      if (!subdomains)
        for (int s = lo; s < hi; ++s)
          for (int k = hp.rowptr[s]; k < hp.rowptr[s + 1]; ++k) {
            int c = hp.col[k];
            if (c < lo) hf.push_back(c);
            else if (c >= hi) hb.push_back(c);
          }
      std::sort(hf.begin(), hf.end()); hf.erase(std::unique(hf.begin(), hf.end()), hf.end());
      std::sort(hb.begin(), hb.end()); hb.erase(std::unique(hb.begin(), hb.end()), hb.end());
      hp.maxHalo = std::max(hp.maxHalo, (int)std::max(hf.size(), hb.size()));
      hp.haloFIdx.insert(hp.haloFIdx.end(), hf.begin(), hf.end());
      hp.haloBIdx.insert(hp.haloBIdx.end(), hb.begin(), hb.end());
      hp.haloFPtr[p + 1] = (int)hp.haloFIdx.size();
      hp.haloBPtr[p + 1] = (int)hp.haloBIdx.size();
    }
    // slots need maxHalo, so a second pass
    for (int p = 0; p < hp.nParts; ++p) {
      const int lo = hp.partStart[p], hi = hp.partStart[p + 1];
      const int* f0 = hp.haloFIdx.data() + hp.haloFPtr[p];
      const int* f1 = hp.haloFIdx.data() + hp.haloFPtr[p + 1];
      const int* b0 = hp.haloBIdx.data() + hp.haloBPtr[p];
      const int* b1 = hp.haloBIdx.data() + hp.haloBPtr[p + 1];
      const int zeroSlot = hp.maxRows + hp.maxHalo;
      for (int s = lo; s < hi; ++s)
        for (int k = hp.rowptr[s]; k < hp.rowptr[s + 1]; ++k) {
          int c = hp.col[k];
          int sl;
          if (c >= lo && c < hi) sl = c - lo;
          else if (subdomains) sl = zeroSlot;
          else if (c < lo) sl = hp.maxRows + (int)(std::lower_bound(f0, f1, c) - f0);
          else sl = hp.maxRows + (int)(std::lower_bound(b0, b1, c) - b0);
          hp.slot[k] = (c < s) ? sl : ~sl;
        }
    }
  }

  // ---- 9. compact in-part tables of the processor-local DIC
  hp.locEntStart.assign(1, 0); hp.locMetaStart.assign(1, 0);
  hp.locSrc.clear(); hp.locIdx.clear(); hp.locMeta.clear();
  hp.maxLocEntries = 0; hp.maxLocMeta = 0;
  if (subdomains) {
    hp.locSrc.reserve(2 * (size_t)nI + 8 * (size_t)hp.nParts);
    hp.locIdx.reserve(2 * (size_t)nI + 8 * (size_t)hp.nParts);
    hp.locMeta.reserve((size_t)nC + 4 * (size_t)hp.nParts);
    hp.locEntStart.reserve((size_t)hp.nParts + 1);
    hp.locMetaStart.reserve((size_t)hp.nParts + 1);
    for (int p = 0; p < hp.nParts; ++p) {
      const int lo = hp.partStart[p], hi = hp.partStart[p + 1];
      const size_t e0 = hp.locSrc.size();
      if (hi - lo > 65535) { err = "part too large for the local DIC tables"; return S4G_BAD_ARG; }
      for (int s = lo; s < hi; ++s) {
        const int off = (int)(hp.locSrc.size() - e0);
        int nl = 0, nu = 0;
        for (int k = hp.rowptr[s]; k < hp.rowptr[s + 1]; ++k) {
          const int c = hp.col[k];
          if (c < s && c >= lo) { hp.locSrc.push_back(k); hp.locIdx.push_back((uint16_t)(c - lo)); ++nl; }
        }
        for (int k = hp.rowptr[s + 1] - 1; k >= hp.rowptr[s]; --k) {
          const int c = hp.col[k];
          if (c > s && c < hi) { hp.locSrc.push_back(k); hp.locIdx.push_back((uint16_t)(c - lo)); ++nu; }
        }
        if (off > 65535 || nl > 255 || nu > 255) {
          err = "part too large for the local DIC tables; use a smaller part_size";
          return S4G_BAD_ARG;
        }
        hp.locMeta.push_back((uint32_t)off | ((uint32_t)nl << 16) | ((uint32_t)nu << 24));
      }
      while ((hp.locSrc.size() - e0) % 8) { hp.locSrc.push_back(-1); hp.locIdx.push_back(0); }
      while (hp.locMeta.size() % 4) hp.locMeta.push_back(0);
      hp.locEntStart.push_back((int)hp.locSrc.size());
      hp.locMetaStart.push_back((int)hp.locMeta.size());
      hp.maxLocEntries = std::max(hp.maxLocEntries, hp.locEntStart[p + 1] - hp.locEntStart[p]);
      hp.maxLocMeta = std::max(hp.maxLocMeta, hp.locMetaStart[p + 1] - hp.locMetaStart[p]);
    }
    // Fixed slots: where every row has at most 3 lower and 3 upper in-part
    // entries (hexahedral meshes in the orders built here), each row gets
    // exactly 3 + 3 slots -- the same entries in the same order, padded with
    // a zero coefficient on a zero row (local index maxRows) -- so that a
    // level walk finds a row's entries at 6 r + (0 | 3) without metadata.
    bool slots = true;
    for (size_t k = 0; k < hp.locMeta.size() && slots; ++k)
      if (((hp.locMeta[k] >> 16) & 0xff) > 3 || (hp.locMeta[k] >> 24) > 3) slots = false;
    if (slots && hp.maxRows >= 65535) slots = false;
    hp.locSlots = slots;
    if (slots) {
      std::vector<int> src, est(1, 0);
      std::vector<uint16_t> idx;
      src.reserve(6 * (size_t)nC + 8 * (size_t)hp.nParts);
      idx.reserve(6 * (size_t)nC + 8 * (size_t)hp.nParts);
      est.reserve((size_t)hp.nParts + 1);
      hp.maxLocEntries = 0;
      for (int p = 0; p < hp.nParts; ++p) {
        const int lo = hp.partStart[p], hi = hp.partStart[p + 1];
        const size_t e0 = src.size();
        const int* gs = hp.locSrc.data() + hp.locEntStart[p];
        const uint16_t* gi = hp.locIdx.data() + hp.locEntStart[p];
        const uint32_t* gm = hp.locMeta.data() + hp.locMetaStart[p];
        for (int r = 0; r < hi - lo; ++r) {
          const int off = (int)(gm[r] & 0xffff), nl = (gm[r] >> 16) & 0xff, nu = gm[r] >> 24;
          for (int u = 0; u < 3; ++u) {
            src.push_back(u < nl ? gs[off + u] : -1);
            idx.push_back(u < nl ? gi[off + u] : (uint16_t)hp.maxRows);
          }
          for (int u = 0; u < 3; ++u) {
            src.push_back(u < nu ? gs[off + nl + u] : -1);
            idx.push_back(u < nu ? gi[off + nl + u] : (uint16_t)hp.maxRows);
          }
        }
        while ((src.size() - e0) % 8) { src.push_back(-1); idx.push_back((uint16_t)hp.maxRows); }
        est.push_back((int)src.size());
        hp.maxLocEntries = std::max(hp.maxLocEntries, est[p + 1] - est[p]);
      }
      hp.locSrc.swap(src);
      hp.locIdx.swap(idx);
      hp.locEntStart.swap(est);
      hp.locMeta.clear();
      hp.locMetaStart.assign(hp.nParts + 1, 0);
      hp.maxLocMeta = 0;
    }
    hp.locDesc.resize(8 * (size_t)hp.nParts);
    for (int p = 0; p < hp.nParts; ++p) {
      int* d8 = hp.locDesc.data() + 8 * (size_t)p;
      d8[0] = hp.partStart[p]; d8[1] = hp.partStart[p + 1] - hp.partStart[p];
      d8[2] = hp.locEntStart[p]; d8[3] = hp.locEntStart[p + 1] - hp.locEntStart[p];
      d8[4] = hp.locMetaStart[p]; d8[5] = hp.locMetaStart[p + 1] - hp.locMetaStart[p];
      d8[6] = hp.lvlOff[p]; d8[7] = hp.lvlOff[p + 1] - hp.lvlOff[p];
    }
  }
  return S4G_OK;
}

}  // namespace s4g

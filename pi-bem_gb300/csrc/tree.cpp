// Octree, interaction lists and operator plan of the FMM-BEM operator.
//
// The box set, the leaf rule and the three lists reproduce pi-BEM's
// BEMFMA::generate_octree_blocking (source/bem_fma.cc:3615-4801) exactly:
//   * root cube pMin = -1.1 max|x_i|, side 2.2 max|x_i| (bem_fma.cc:3713-3718);
//   * level-by-level 8-way split in the child order (0,0,0),(1,0,0),(1,1,0),
//     (0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1), points on a split plane going
//     low (bem_fma.cc:3811-3973);
//   * a box exists iff it holds nodes or quadrature points (bem_fma.cc:3975);
//   * childless iff round(sum 1/|double set|) <= leaf size (bem_fma.cc:4135);
//   * near neighbours by the TOLL touch test (bem_fma.cc:4269-4580);
//   * intList = near neighbours + boxes of the quadrature points of the cells
//     around the box's nodes and their doubles (bem_fma.cc:4612-4668);
//   * nonIntList from the parent's (or previous sublevel's) intList
//     (bem_fma.cc:4669-4711).
// The implementation is data-parallel instead of std::set based: every point
// gets its full path key by the reference's own floating-point comparisons,
// points are sorted by key, and the boxes of a level are the runs of equal
// key prefixes inside the ranges of the previous level's parents, which
// yields the reference's breadth-first box numbering.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <numeric>
#include <unordered_map>

#include "pibem_internal.h"

namespace pibem
{
  namespace
  {
    constexpr double TOLL = 0.001; // source/bem_fma.cc:1
    const int child_off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                 {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    const int digit_of[2][2][2] = {{{0, 1}, {3, 2}}, {{4, 5}, {7, 6}}}; // [hz][hy][hx]

    inline int digit_at(uint64_t key, int L, int l) { return int((key >> (3 * (L - l))) & 7u); }

    bool touches(const Tree &t, int a, int b)
    {
      double PMin1[3], PMax1[3], PMin2[3], PMax2[3];
      for (int k = 0; k < 3; ++k)
        {
          PMin1[k] = t.pmin[3 * a + k];
          PMax1[k] = 2. * (t.delta[a] / 2.) + PMin1[k];
          PMin2[k] = t.pmin[3 * b + k];
          PMax2[k] = 2. * (t.delta[b] / 2.) + PMin2[k];
        }
      for (int ax = 0; ax < 3; ++ax)
        {
          int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
          if ((std::fabs(PMin1[ax] - PMax2[ax]) <= TOLL) ||
              (std::fabs(PMax1[ax] - PMin2[ax]) <= TOLL))
            if ((PMin1[o1] - TOLL <= PMax2[o1]) && (PMax1[o1] + TOLL >= PMin2[o1]))
              if ((PMin1[o2] - TOLL <= PMax2[o2]) && (PMax1[o2] + TOLL >= PMin2[o2]))
                return true;
        }
      return false;
    }

    void sort_unique(std::vector<int> &v)
    {
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
    }
  } // namespace

  void build_tree(const MeshHost &mesh, const std::vector<double> &qpts, int nq, int L,
                  int max_nodes, Tree &t)
  {
    const int64_t N = mesh.n_nodes;
    const int64_t Q = int64_t(qpts.size() / 3);
    if (L < 1 || L > 20)
      throw Error(PIBEM_EINVAL, "Number of Octree Levels must be in 1..20");
    t     = Tree();
    t.L   = L;
    double max_coor = 0;
    for (int64_t i = 0; i < 3 * N; ++i)
      max_coor = std::max(max_coor, std::fabs(mesh.xyz[i]));
    const double p0     = -1.1 * max_coor;
    const double delta0 = 2.2 * max_coor;

    // Path keys with the reference's comparisons (bem_fma.cc:3844-3973).
    auto key_of = [&](const double *x) {
      double   pm[3] = {p0, p0, p0};
      double   d     = delta0;
      uint64_t k     = 0;
      for (int l = 1; l <= L; ++l)
        {
          d /= 2.;
          bool hx = !(x[0] <= pm[0] + d);
          bool hy = !(x[1] <= pm[1] + d);
          bool hz = !(x[2] <= pm[2] + d);
          k       = (k << 3) | uint64_t(digit_of[hz][hy][hx]);
          if (hx)
            pm[0] = pm[0] + d;
          if (hy)
            pm[1] = pm[1] + d;
          if (hz)
            pm[2] = pm[2] + d;
        }
      return k;
    };
    std::vector<std::pair<uint64_t, int>> nk(N), qk(Q);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i)
      nk[i] = {key_of(&mesh.xyz[3 * i]), int(i)};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < Q; ++i)
      qk[i] = {key_of(&qpts[3 * i]), int(i)};
    std::sort(nk.begin(), nk.end());
    std::sort(qk.begin(), qk.end());
    std::vector<uint64_t> nkey(N), qkey(Q);
    t.node_sorted.resize(N);
    t.quad_sorted.resize(Q);
    for (int64_t i = 0; i < N; ++i)
      {
        nkey[i]          = nk[i].first;
        t.node_sorted[i] = nk[i].second;
      }
    for (int64_t i = 0; i < Q; ++i)
      {
        qkey[i]          = qk[i].first;
        t.quad_sorted[i] = qk[i].second;
      }
    nk.clear();
    nk.shrink_to_fit();
    qk.clear();
    qk.shrink_to_fit();

    auto new_box = [&](int lvl, int par, int dg, const double *pm, double d, const int *icp,
                       int nb0, int nb1, int qb0, int qb1) {
      t.level.push_back(lvl);
      t.parent.push_back(par);
      t.nchild.push_back(0);
      t.child_first.push_back(-1);
      t.digit.push_back(dg);
      for (int k = 0; k < 3; ++k)
        {
          t.pmin.push_back(pm[k]);
          t.ic.push_back(icp[k]);
        }
      t.delta.push_back(d);
      t.nbeg.push_back(nb0);
      t.nend.push_back(nb1);
      t.qbeg.push_back(qb0);
      t.qend.push_back(qb1);
      return int(t.level.size()) - 1;
    };
    {
      double pm[3] = {p0, p0, p0};
      int    ic0[3] = {0, 0, 0};
      new_box(0, 0, 0, pm, delta0, ic0, 0, int(N), 0, int(Q));
    }
    t.startLevel.assign(L + 1, 0);
    t.endLevel.assign(L + 1, 0);
    t.dofs_filled.assign(L + 1, {});
    std::vector<int> parents = {0};
    double           d       = delta0;
    std::vector<double> weight(N);
    for (int64_t i = 0; i < N; ++i)
      weight[i] = 1.0 / double(mesh.dbl_off[i + 1] - mesh.dbl_off[i]);

    for (int l = 1; l <= L; ++l)
      {
        d /= 2.;
        for (int P : parents)
          {
            int na = t.nbeg[P], qa = t.qbeg[P];
            for (int dg = 0; dg < 8; ++dg)
              {
                int ne = na, qe = qa;
                while (ne < t.nend[P] && digit_at(nkey[ne], L, l) == dg)
                  ++ne;
                while (qe < t.qend[P] && digit_at(qkey[qe], L, l) == dg)
                  ++qe;
                if (ne > na || qe > qa)
                  {
                    double pm[3];
                    int    icc[3];
                    for (int k = 0; k < 3; ++k)
                      {
                        pm[k]  = child_off[dg][k] ? t.pmin[3 * P + k] + d : t.pmin[3 * P + k];
                        icc[k] = 2 * t.ic[3 * P + k] + child_off[dg][k];
                      }
                    int id = new_box(l, P, dg, pm, d, icc, na, ne, qa, qe);
                    if (t.nchild[P] == 0)
                      t.child_first[P] = id;
                    t.nchild[P]++;
                  }
                na = ne;
                qa = qe;
              }
          }
        t.startLevel[l] = t.endLevel[l - 1] + 1;
        t.endLevel[l]   = int(t.level.size()) - 1;
        std::vector<int> next;
        for (int b = t.startLevel[l]; b <= t.endLevel[l]; ++b)
          {
            // sum in ascending node order, as the reference's node list
            std::vector<int> ids(t.node_sorted.begin() + t.nbeg[b], t.node_sorted.begin() + t.nend[b]);
            std::sort(ids.begin(), ids.end());
            double numNodes = 0.0;
            for (int i : ids)
              numNodes += weight[i];
            if (std::round(numNodes) <= max_nodes)
              t.childless.push_back(b);
            else
              next.push_back(b);
            if (numNodes > 0)
              t.dofs_filled[l].push_back(b);
          }
        parents.swap(next);
      }
    for (int b : parents)
      t.childless.push_back(b);
    t.nb = int(t.level.size());
    t.is_childless.assign(t.nb, 0);
    for (int b : t.childless)
      t.is_childless[b] = 1;

    // box of every quad point at every level (leaf box below its level)
    t.qbox.assign(size_t(L + 1) * Q, 0);
    for (int b = 0; b < t.nb; ++b)
      {
        int lb = t.level[b];
        int lmax = t.nchild[b] == 0 ? L : lb;
        for (int k = t.qbeg[b]; k < t.qend[b]; ++k)
          {
            int q = t.quad_sorted[k];
            for (int j = lb; j <= lmax; ++j)
              t.qbox[size_t(j) * Q + q] = b;
          }
      }
    t.node_leaf.assign(N, -1);
    for (int b : t.childless)
      for (int k = t.nbeg[b]; k < t.nend[b]; ++k)
        t.node_leaf[t.node_sorted[k]] = b;

    // ---- near neighbours (bem_fma.cc:4269-4580)
    t.nn.assign(t.nb, std::vector<std::vector<int>>(1));
    t.il.assign(t.nb, std::vector<std::vector<int>>(1));
    t.nil.assign(t.nb, std::vector<std::vector<int>>(1));
    std::vector<int> lvl1;
    for (int b = t.startLevel[1]; b <= t.endLevel[1]; ++b)
      lvl1.push_back(b);
    for (int b : lvl1)
      {
        t.nn[b][0] = lvl1;
        t.il[b][0] = lvl1;
      }
    for (int l = 2; l <= L; ++l)
      {
#pragma omp parallel for schedule(dynamic, 16)
        for (int b = t.startLevel[l]; b <= t.endLevel[l]; ++b)
          {
            std::vector<int> cand = {b};
            for (int pos : t.nn[t.parent[b]][0])
              {
                if (t.nchild[pos] == 0 && touches(t, b, pos))
                  cand.push_back(pos);
                for (int c = 0; c < t.nchild[pos]; ++c)
                  if (touches(t, b, t.child_first[pos] + c))
                    cand.push_back(t.child_first[pos] + c);
              }
            sort_unique(cand);
            t.nn[b][0] = cand;
            if (t.nchild[b] == 0)
              {
                int ns = L - l + 1;
                t.nn[b].resize(ns);
                t.il[b].resize(ns);
                t.nil[b].resize(ns);
                for (int sub = 1; sub < ns; ++sub)
                  {
                    std::vector<int> c2;
                    for (int pos : t.nn[b][sub - 1])
                      {
                        if (t.nchild[pos] == 0)
                          c2.push_back(pos);
                        for (int c = 0; c < t.nchild[pos]; ++c)
                          if (touches(t, b, t.child_first[pos] + c))
                            c2.push_back(t.child_first[pos] + c);
                      }
                    sort_unique(c2);
                    t.nn[b][sub] = c2;
                  }
              }
          }
      }

    // ---- interaction and non-interaction lists (bem_fma.cc:4588-4711)
    for (int l = 2; l <= L; ++l)
      {
#pragma omp parallel for schedule(dynamic, 16)
        for (int b = t.startLevel[l]; b <= t.endLevel[l]; ++b)
          {
            std::vector<int> cells;
            for (int k = t.nbeg[b]; k < t.nend[b]; ++k)
              {
                int node = t.node_sorted[k];
                for (int a = mesh.dbl_off[node]; a < mesh.dbl_off[node + 1]; ++a)
                  {
                    int dn = mesh.dbl_ids[a];
                    for (int e = mesh.elem_off[dn]; e < mesh.elem_off[dn + 1]; ++e)
                      cells.push_back(mesh.elem_ids[e]);
                  }
              }
            sort_unique(cells);
            const int ns = int(t.nn[b].size());
            for (int sub = 0; sub < ns; ++sub)
              {
                std::vector<int> v = t.nn[b][sub];
                const int       *qb = &t.qbox[size_t(l + sub) * Q];
                for (int c : cells)
                  for (int q = 0; q < nq; ++q)
                    v.push_back(qb[size_t(c) * nq + q]);
                sort_unique(v);
                t.il[b][sub] = v;
              }
            for (int sub = 0; sub < ns; ++sub)
              {
                const std::vector<int> &il  = t.il[b][sub];
                const std::vector<int> &pil = sub == 0 ? t.il[t.parent[b]][0] : t.il[b][sub - 1];
                std::vector<int>        out;
                for (int pos : pil)
                  {
                    if (t.nchild[pos] == 0)
                      {
                        if (!std::binary_search(il.begin(), il.end(), pos))
                          out.push_back(pos);
                      }
                    else
                      for (int c = 0; c < t.nchild[pos]; ++c)
                        {
                          int cid = t.child_first[pos] + c;
                          if (!std::binary_search(il.begin(), il.end(), cid))
                            out.push_back(cid);
                        }
                  }
                sort_unique(out);
                t.nil[b][sub] = out;
              }
          }
      }
  }

  void mirror_mesh(int64_t n_nodes, const double *xyz, int64_t n_cells, const int32_t *cells,
                   const std::vector<std::vector<int32_t>> &sets, bool double_body, double z0,
                   MeshHost &m)
  {
    const int64_t f = double_body ? 2 : 1;
    m.n_dofs        = n_nodes;
    m.n_cells_body  = n_cells;
    m.n_nodes       = f * n_nodes;
    m.n_cells       = f * n_cells;
    m.xyz.assign(xyz, xyz + 3 * n_nodes);
    m.cells.assign(cells, cells + 4 * n_cells);
    m.dbl_off.assign(m.n_nodes + 1, 0);
    m.dbl_ids.clear();
    for (int64_t i = 0; i < n_nodes; ++i)
      {
        m.dbl_ids.insert(m.dbl_ids.end(), sets[i].begin(), sets[i].end());
        m.dbl_off[i + 1] = int32_t(m.dbl_ids.size());
      }
    if (!double_body)
      return;
    const int32_t o = int32_t(n_nodes);
    for (int64_t i = 0; i < n_nodes; ++i)
      {
        m.xyz.push_back(xyz[3 * i]);
        m.xyz.push_back(xyz[3 * i + 1]);
        m.xyz.push_back(2.0 * z0 - xyz[3 * i + 2]);
      }
    // lexicographic (v0, v1, v2, v3) -> (v0, v2, v1, v3): the reference
    // coordinates swap, which turns the normal of the reflected cell around
    for (int64_t c = 0; c < n_cells; ++c)
      {
        const int32_t *v = cells + 4 * c;
        m.cells.push_back(v[0] + o);
        m.cells.push_back(v[2] + o);
        m.cells.push_back(v[1] + o);
        m.cells.push_back(v[3] + o);
      }
    for (int64_t i = 0; i < n_nodes; ++i)
      {
        for (int32_t d : sets[i])
          m.dbl_ids.push_back(d + o);
        m.dbl_off[n_nodes + i + 1] = int32_t(m.dbl_ids.size());
      }
  }

  void build_plan(const MeshHost &mesh, const Tree &t, int nq, int p, Plan &pl, int chunk_pairs)
  {
    pl     = Plan();
    pl.p   = p;
    pl.K   = (p + 1) * (p + 1);
    const int64_t Q = int64_t(t.qbox.size() / (t.L + 1));
    // Target boxes: boxes holding collocation nodes (every box with nodes for
    // one body; a double body's boxes of image nodes only are sources only).
    std::vector<char> tgt(t.nb, 0);
    for (int b = 0; b < t.nb; ++b)
      for (int k = t.nbeg[b]; k < t.nend[b] && !tgt[b]; ++k)
        tgt[b] = t.node_sorted[k] < mesh.n_dofs;
    std::vector<std::vector<int>> tfill(t.L + 1);
    for (int l = 0; l <= t.L; ++l)
      for (int b : t.dofs_filled[l])
        if (tgt[b])
          tfill[l].push_back(b);

    // cell -> quad mask of a set of boxes
    // cell -> quad mask of a set of boxes, sorted by cell: a dense per-thread
    // mask array over the cells (zero between calls) and the list of the
    // cells it touched
    const int64_t n_qcells = nq > 0 ? int64_t(t.quad_sorted.size()) / nq : 0;
    struct CollectScratch
    {
      std::vector<uint64_t> mask;
      std::vector<int>      touched;
    };
    auto collect = [&](const std::vector<int> &boxes, std::vector<std::pair<int, uint64_t>> &out,
                       CollectScratch &sc) {
      if (int64_t(sc.mask.size()) < n_qcells)
        sc.mask.assign(n_qcells, 0);
      sc.touched.clear();
      for (int bx : boxes)
        for (int k = t.qbeg[bx]; k < t.qend[bx]; ++k)
          {
            const int qid = t.quad_sorted[k], c = qid / nq;
            if (!sc.mask[c])
              sc.touched.push_back(c);
            sc.mask[c] |= uint64_t(1) << (qid % nq);
          }
      std::sort(sc.touched.begin(), sc.touched.end());
      out.clear();
      out.reserve(sc.touched.size());
      for (int c : sc.touched)
        {
          out.push_back({c, sc.mask[c]});
          sc.mask[c] = 0;
        }
    };

    // coarse non-interaction boxes (direct integration, bem_fma.cc:997-1153)
    std::vector<std::vector<std::pair<int, uint64_t>>> coarse(t.nb);
    for (int l = 1; l <= t.L; ++l)
      {
        const std::vector<int> &fl = tfill[l];
#pragma omp parallel
        {
          CollectScratch sc;
#pragma omp for schedule(dynamic, 16)
          for (int k = 0; k < int(fl.size()); ++k)
            {
              int              b = fl[k];
              std::vector<int> boxes;
              for (size_t sub = 0; sub < t.nn[b].size(); ++sub)
                for (int pos : t.nil[b][sub])
                  if (pos < t.startLevel[l])
                    boxes.push_back(pos);
              sort_unique(boxes);
              if (!boxes.empty())
                collect(boxes, coarse[b], sc);
            }
        }
      }

    // ---- near field per childless box with nodes
    std::vector<int> nleaves;
    for (int b : t.childless)
      if (tgt[b])
        nleaves.push_back(b);
    const int nl = int(nleaves.size());
    std::vector<std::vector<int>>       rows(nl), cols(nl);
    std::vector<std::vector<NearEntry>> ents(nl);
    std::vector<std::vector<int>>       gptr(nl), gids(nl);
#pragma omp parallel
    {
    CollectScratch sc;
#pragma omp for schedule(dynamic, 8)
    for (int k = 0; k < nl; ++k)
      {
        int                                    b = nleaves[k];
        std::vector<std::pair<int, uint64_t>> e1;
        collect(t.il[b].back(), e1, sc);
        std::vector<NearEntry> E;
        for (auto &cm : e1)
          E.push_back(NearEntry{cm.first, 1, cm.second, {0, 0, 0, 0}});
        // ancestors (and the box itself) from level 1 down
        std::vector<int> chain;
        for (int a = b; t.level[a] >= 1; a = t.parent[a])
          chain.push_back(a);
        std::reverse(chain.begin(), chain.end());
        for (int a : chain)
          for (auto &cm : coarse[a])
            E.push_back(NearEntry{cm.first, 0, cm.second, {0, 0, 0, 0}});
        // columns: the unknowns (an image node's column is its original's)
        std::vector<int> c;
        for (auto &e : E)
          for (int j = 0; j < 4; ++j)
            c.push_back(mesh.dof(mesh.cells[4 * size_t(e.cell) + j]));
        sort_unique(c);
        for (auto &e : E)
          for (int j = 0; j < 4; ++j)
            e.lcol[j] = int(std::lower_bound(c.begin(), c.end(),
                                             mesh.dof(mesh.cells[4 * size_t(e.cell) + j])) -
                            c.begin());
        // per column, the (entry, vertex) ids e * 4 + j touching it, in
        // ascending order (a counting sort over the columns)
        std::vector<int> gp(c.size() + 1, 0), gi(E.size() * 4);
        for (size_t ei = 0; ei < E.size(); ++ei)
          for (int j = 0; j < 4; ++j)
            ++gp[E[ei].lcol[j] + 1];
        for (size_t q = 0; q < c.size(); ++q)
          gp[q + 1] += gp[q];
        {
          std::vector<int> at(gp.begin(), gp.end() - 1);
          for (size_t ei = 0; ei < E.size(); ++ei)
            for (int j = 0; j < 4; ++j)
              gi[at[E[ei].lcol[j]]++] = int(ei) * 4 + j;
        }
        std::vector<int> r;
        for (int s = t.nbeg[b]; s < t.nend[b]; ++s)
          if (t.node_sorted[s] < mesh.n_dofs)
            r.push_back(t.node_sorted[s]);
        std::sort(r.begin(), r.end());
        rows[k] = std::move(r);
        cols[k] = std::move(c);
        ents[k] = std::move(E);
        gptr[k] = std::move(gp);
        gids[k] = std::move(gi);
      }
    }
    pl.nleaf_box = nleaves;
    pl.nrow_ptr.assign(nl + 1, 0);
    pl.ncol_ptr.assign(nl + 1, 0);
    pl.nent_ptr.assign(nl + 1, 0);
    pl.nval_ptr.assign(nl + 1, 0);
    for (int k = 0; k < nl; ++k)
      {
        pl.nrow_ptr[k + 1] = pl.nrow_ptr[k] + int64_t(rows[k].size());
        pl.ncol_ptr[k + 1] = pl.ncol_ptr[k] + int64_t(cols[k].size());
        pl.nent_ptr[k + 1] = pl.nent_ptr[k] + int64_t(ents[k].size());
        // rows padded to a multiple of 4 values (16-byte vector loads)
        pl.nval_ptr[k + 1] = pl.nval_ptr[k] + int64_t(rows[k].size()) * ((int64_t(cols[k].size()) + 3) / 4 * 4);
      }
    // the leaves' pieces concatenated in leaf order (offsets first, then the
    // copies in parallel); gather_ptr per column (global column position),
    // gather ids local to the leaf
    std::vector<int64_t> gid_ptr(nl + 1, 0);
    for (int k = 0; k < nl; ++k)
      gid_ptr[k + 1] = gid_ptr[k] + int64_t(gids[k].size());
    pl.nrows.resize(pl.nrow_ptr[nl]);
    pl.row_leaf.resize(pl.nrow_ptr[nl]);
    pl.ncols.resize(pl.ncol_ptr[nl]);
    pl.entries.resize(pl.nent_ptr[nl]);
    pl.gather_ptr.resize(pl.ncol_ptr[nl] + 1);
    pl.gather_ids.resize(gid_ptr[nl]);
#pragma omp parallel for schedule(dynamic, 64)
    for (int k = 0; k < nl; ++k)
      {
        std::copy(rows[k].begin(), rows[k].end(), pl.nrows.begin() + pl.nrow_ptr[k]);
        std::fill(pl.row_leaf.begin() + pl.nrow_ptr[k], pl.row_leaf.begin() + pl.nrow_ptr[k + 1], k);
        std::copy(cols[k].begin(), cols[k].end(), pl.ncols.begin() + pl.ncol_ptr[k]);
        std::copy(ents[k].begin(), ents[k].end(), pl.entries.begin() + pl.nent_ptr[k]);
        for (size_t c = 0; c < cols[k].size(); ++c)
          pl.gather_ptr[pl.ncol_ptr[k] + int64_t(c)] = int(gid_ptr[k]) + gptr[k][c];
        std::copy(gids[k].begin(), gids[k].end(), pl.gather_ids.begin() + gid_ptr[k]);
      }
    pl.gather_ptr[pl.ncol_ptr[nl]] = int(gid_ptr[nl]);

    // ---- P2M tables per childless box with quadrature points
    std::vector<int> pleaves;
    for (int b : t.childless)
      if (t.qend[b] > t.qbeg[b])
        pleaves.push_back(b);
    const int np = int(pleaves.size());
    std::vector<std::vector<int>> prow(np), pcp(np), pcq(np);
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < np; ++k)
      {
        int                                b = pleaves[k];
        std::vector<std::pair<int, int>> dq; // (dof, qid*4+j)
        for (int s = t.qbeg[b]; s < t.qend[b]; ++s)
          {
            int qid = t.quad_sorted[s];
            int c   = qid / nq;
            for (int j = 0; j < 4; ++j)
              dq.push_back({mesh.dof(mesh.cells[4 * size_t(c) + j]), qid * 4 + j});
          }
        std::sort(dq.begin(), dq.end());
        std::vector<int> rws, cp(1, 0), cq;
        for (size_t i = 0; i < dq.size(); ++i)
          {
            if (i == 0 || dq[i].first != dq[i - 1].first)
              {
                if (i > 0)
                  cp.push_back(int(cq.size()));
                rws.push_back(dq[i].first);
              }
            cq.push_back(dq[i].second);
          }
        cp.push_back(int(cq.size()));
        prow[k] = std::move(rws);
        pcp[k]  = std::move(cp);
        pcq[k]  = std::move(cq);
      }
    pl.pleaf_box = pleaves;
    pl.prow_ptr.assign(np + 1, 0);
    std::vector<int64_t> pq_ptr(np + 1, 0);
    for (int k = 0; k < np; ++k)
      {
        pl.prow_ptr[k + 1] = pl.prow_ptr[k] + int64_t(prow[k].size());
        pq_ptr[k + 1]      = pq_ptr[k] + int64_t(pcq[k].size());
      }
    pl.prow_dof.resize(pl.prow_ptr[np]);
    pl.pcontrib_ptr.resize(pl.prow_ptr[np] + 1);
    pl.pcontrib_q.resize(pq_ptr[np]);
    pl.pcontrib_ptr[0] = 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int k = 0; k < np; ++k)
      {
        std::copy(prow[k].begin(), prow[k].end(), pl.prow_dof.begin() + pl.prow_ptr[k]);
        for (size_t r = 0; r < prow[k].size(); ++r)
          pl.pcontrib_ptr[pl.prow_ptr[k] + int64_t(r) + 1] = pq_ptr[k] + pcp[k][r + 1];
        std::copy(pcq[k].begin(), pcq[k].end(), pl.pcontrib_q.begin() + pq_ptr[k]);
      }

    // ---- L2P per childless box with nodes (same leaves as the near field)
    pl.lleaf_box = nleaves;
    pl.lnode_ptr = pl.nrow_ptr;
    pl.lnode_ids = pl.nrows;

    // ---- M2L / M2P pairs, per level over boxes with nodes (bem_fma.cc:2582-2704)
    std::unordered_map<int64_t, int> offid;
    auto off_key = [](int dx, int dy, int dz) {
      return (int64_t(dx + 1048576) << 42) | (int64_t(dy + 1048576) << 21) | int64_t(dz + 1048576);
    };
    pl.m2l_tgt_ptr_level.assign(t.L + 2, 0);
    pl.m2l_src_ptr.push_back(0);
    pl.m2p_src_ptr.push_back(0);
    for (int l = 1; l <= t.L; ++l)
      {
        pl.m2l_tgt_ptr_level[l] = int(pl.m2l_tgt.size());
        const int sL = t.startLevel[l], eL = t.endLevel[l];
        for (int b : tfill[l])
          {
            std::vector<int> ms, mp;
            for (size_t sub = 0; sub < t.nn[b].size(); ++sub)
              for (int pos : t.nil[b][sub])
                {
                  if (pos < sL)
                    continue;
                  if (pos <= eL)
                    ms.push_back(pos);
                  else
                    mp.push_back(pos);
                }
            if (!ms.empty())
              {
                pl.m2l_tgt.push_back(b);
                for (int s : ms)
                  {
                    int dx = t.ic[3 * s] - t.ic[3 * b], dy = t.ic[3 * s + 1] - t.ic[3 * b + 1],
                        dz = t.ic[3 * s + 2] - t.ic[3 * b + 2];
                    int64_t key = off_key(dx, dy, dz);
                    auto    it  = offid.find(key);
                    int     id;
                    if (it == offid.end())
                      {
                        id = int(pl.offsets.size() / 3);
                        offid[key] = id;
                        pl.offsets.push_back(dx);
                        pl.offsets.push_back(dy);
                        pl.offsets.push_back(dz);
                      }
                    else
                      id = it->second;
                    pl.m2l_src.push_back(s);
                    pl.m2l_off.push_back(id);
                  }
                pl.m2l_src_ptr.push_back(int64_t(pl.m2l_src.size()));
              }
            if (!mp.empty())
              {
                pl.m2p_tgt.push_back(b);
                pl.m2p_src.insert(pl.m2p_src.end(), mp.begin(), mp.end());
                pl.m2p_src_ptr.push_back(int64_t(pl.m2p_src.size()));
              }
          }
      }
    pl.m2l_tgt_ptr_level[t.L + 1] = int(pl.m2l_tgt.size());
    pl.n_m2l = int64_t(pl.m2l_src.size());
    pl.n_m2p = int64_t(pl.m2p_src.size());
    // ---- batched translation pairs
    {
      const int noff = int(pl.offsets.size() / 3);
      // chunk helper: pairs already grouped by operator in [a, b)
      auto cut = [&](int64_t a, int64_t b) {
        int64_t i = a;
        while (i < b)
          {
            int64_t j = i;
            while (j < b && pl.q_op[j] == pl.q_op[i] && j - i < chunk_pairs)
              ++j;
            pl.ch_start.push_back(int32_t(i));
            pl.ch_cnt.push_back(int32_t(j - i));
            pl.ch_op.push_back(pl.q_op[i]);
            i = j;
          }
      };
      // M2L pairs of all levels, grouped by offset (stable)
      const int64_t        np = pl.n_m2l;
      std::vector<int64_t> cnt(noff + 1, 0);
      for (int64_t e = 0; e < np; ++e)
        cnt[pl.m2l_off[e] + 1]++;
      for (int o = 0; o < noff; ++o)
        cnt[o + 1] += cnt[o];
      std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1), qof(np);
      pl.q_src.assign(np, 0);
      pl.q_op.assign(np, 0);
      for (int64_t e = 0; e < np; ++e)
        {
          int64_t q   = pos[pl.m2l_off[e]]++;
          qof[e]      = q;
          pl.q_src[q] = pl.m2l_src[e];
          pl.q_op[q]  = pl.m2l_off[e];
        }
      cut(0, np);
      pl.m2l_chunk_end = int(pl.ch_start.size());
      // target-major slot of each M2L pair (its place in m2l_src)
      pl.m2l_yslot.assign(np, 0);
      for (int64_t e = 0; e < np; ++e)
        pl.m2l_yslot[qof[e]] = int32_t(e);
      // Levels whose expansions are ever read: multipoles of the boxes at or
      // below the shallowest M2L / M2P source (M2M stops there), locals of
      // the boxes at or below the shallowest M2L target (above it they are
      // zero: no L2L from there, the boxes with nodes get a zero expansion).
      int lo_src = t.L + 1, lo_tgt = t.L + 1;
      for (int32_t b : pl.m2l_src)
        lo_src = std::min(lo_src, t.level[b]);
      for (int32_t b : pl.m2p_src)
        lo_src = std::min(lo_src, t.level[b]);
      for (int32_t b : pl.m2l_tgt)
        lo_tgt = std::min(lo_tgt, t.level[b]);
      // M2M: children at level l -> parents at level l-1, grouped by octant
      pl.up_chunk_ptr.assign(t.L + 2, 0);
      pl.up_box_ptr.assign(t.L + 2, 0);
      pl.up_q_ptr.push_back(0);
      std::vector<int64_t> child_q(t.nb, -1);
      for (int l = 1; l <= t.L; ++l)
        {
          pl.up_chunk_ptr[l] = int(pl.ch_start.size());
          pl.up_box_ptr[l]   = int(pl.up_box.size());
          if (l - 1 < lo_src)
            continue;
          int64_t q0 = int64_t(pl.q_src.size());
          for (int dg = 0; dg < 8; ++dg)
            for (int b = t.startLevel[l]; b <= t.endLevel[l] && t.startLevel[l] <= t.endLevel[l]; ++b)
              if (t.digit[b] == dg)
                {
                  child_q[b] = int64_t(pl.q_src.size());
                  pl.q_src.push_back(b);
                  pl.q_op.push_back(noff + dg);
                }
          cut(q0, int64_t(pl.q_src.size()));
          // parents (level l-1) gather their children's products
          for (int P = t.startLevel[l - 1]; P <= t.endLevel[l - 1]; ++P)
            if (t.nchild[P] > 0)
              {
                pl.up_box.push_back(P);
                const size_t at = pl.up_child8.size();
                pl.up_child8.resize(at + 8, -1);
                for (int c = 0; c < t.nchild[P]; ++c)
                  {
                    const int cb = t.child_first[P] + c;
                    pl.up_q.push_back(int32_t(child_q[cb]));
                    pl.up_child8[at + t.digit[cb]] = cb;
                  }
                pl.up_q_ptr.push_back(int64_t(pl.up_q.size()));
              }
        }
      pl.up_chunk_ptr[t.L + 1] = int(pl.ch_start.size());
      pl.up_box_ptr[t.L + 1]   = int(pl.up_box.size());
      // L2L: parent (level l-1 >= lo_tgt) -> child with nodes (level l), by
      // octant; gather per box with nodes, listed by octant: its L2L product,
      // then its M2L products.  Boxes with nodes above lo_tgt are listed (with
      // nothing to sum) at the first level that has any.
      pl.down_chunk_ptr.assign(t.L + 2, 0);
      pl.down_box_ptr.assign(t.L + 2, 0);
      pl.down_q_ptr.push_back(0);
      std::vector<int64_t> l2l_q(t.nb, -1);
      std::vector<int64_t> m2l_first(t.nb, -1);
      for (size_t ti = 0; ti < pl.m2l_tgt.size(); ++ti)
        m2l_first[pl.m2l_tgt[ti]] = int64_t(ti);
      const int zero_level = std::min(std::max(lo_tgt, 1), t.L);
      for (int l = 1; l <= t.L; ++l)
        {
          pl.down_chunk_ptr[l] = int(pl.ch_start.size());
          pl.down_box_ptr[l]   = int(pl.down_box.size());
          if (l < zero_level)
            continue;
          std::vector<int> boxes;
          if (l == zero_level)
            for (int l2 = 1; l2 < l; ++l2)
              boxes.insert(boxes.end(), tfill[l2].begin(), tfill[l2].end());
          std::vector<int> here = tfill[l];
          std::stable_sort(here.begin(), here.end(),
                           [&](int a, int b) { return t.digit[a] < t.digit[b]; });
          int64_t q0 = int64_t(pl.q_src.size());
          if (l >= 2 && l - 1 >= lo_tgt)
            for (int b : here)
              {
                l2l_q[b] = int64_t(pl.q_src.size());
                pl.q_src.push_back(t.parent[b]);
                pl.q_op.push_back(noff + 8 + t.digit[b]);
              }
          cut(q0, int64_t(pl.q_src.size()));
          boxes.insert(boxes.end(), here.begin(), here.end());
          for (int b : boxes)
            {
              pl.down_box.push_back(b);
              pl.down_oct.push_back(uint8_t(t.digit[b] & 7));
              pl.down_par.push_back(l2l_q[b] >= 0 ? t.parent[b] : -1);
              pl.down_m2l_beg.push_back(m2l_first[b] >= 0 ? int32_t(pl.m2l_src_ptr[m2l_first[b]]) : 0);
              pl.down_m2l_end.push_back(m2l_first[b] >= 0 ? int32_t(pl.m2l_src_ptr[m2l_first[b] + 1]) : 0);
              if (l2l_q[b] >= 0)
                pl.down_q.push_back(int32_t(l2l_q[b]));
              if (m2l_first[b] >= 0)
                {
                  int64_t ti = m2l_first[b];
                  for (int64_t e = pl.m2l_src_ptr[ti]; e < pl.m2l_src_ptr[ti + 1]; ++e)
                    pl.down_q.push_back(int32_t(qof[e]));
                }
              pl.down_q_ptr.push_back(int64_t(pl.down_q.size()));
            }
        }
      pl.down_chunk_ptr[t.L + 1] = int(pl.ch_start.size());
      pl.down_box_ptr[t.L + 1]   = int(pl.down_box.size());
    }

    // ---- L2L: boxes with nodes at levels >= 2
    pl.l2l_ptr_level.assign(t.L + 2, 0);
    for (int l = 1; l <= t.L; ++l)
      {
        pl.l2l_ptr_level[l] = int(pl.l2l_box.size());
        if (l >= 2)
          for (int b : tfill[l])
            pl.l2l_box.push_back(b);
      }
    pl.l2l_ptr_level[t.L + 1] = int(pl.l2l_box.size());
    (void)Q;
  }

  // ---------------------------------------------------------------------
  // Real-form translation operators.
  //
  // Expansions are stored as K = (p+1)^2 reals: for each degree n the real part
  // of the m = 0 coefficient followed by (re, im) of m = 1..n.  Coefficients are
  // scaled by the box side h: multipole M^_n = M_n / h^n, local L^_n = L_n h^(n+1),
  // which makes every operator independent of the level.  The complex formulas
  // are pi-BEM's (MultipoleExpansion::Add(child) multipole_expansion.cc:185-261,
  // LocalExpansion::Add(M) local_expansion.cc:180-248, LocalExpansion::Add(L)
  // local_expansion.cc:108-176); each complex term c * a, with a = M^m,
  // conj(M^m) or Re(M^m), is spread onto the real matrix.
  // ---------------------------------------------------------------------
  namespace
  {
    using cplx = std::complex<double>;
    inline int ridx(int n, int m, int part) { return m == 0 ? n * n : n * n + 2 * m - 1 + part; }

    struct Anm
    {
      double a[21][21];
      Anm()
      {
        for (int n = 0; n <= 20; ++n)
          for (int m = 0; m <= n; ++m)
            {
              double f1 = 1., f2 = 1.;
              for (int i = n - m; i > 0; i--)
                f1 *= i;
              for (int i = n + m; i > 0; i--)
                f2 *= i;
              a[n][m] = std::pow(-1., double(n)) / std::sqrt(f1 * f2);
            }
      }
      double operator()(int n, int m) const { return a[n][std::abs(m)]; }
    };
    const Anm &A()
    {
      static Anm t;
      return t;
    }
    inline double re_ipow(int k)
    {
      int r = ((k % 4) + 4) % 4;
      return r == 0 ? 1.0 : (r == 2 ? -1.0 : 0.0);
    }
    // Normalised associated Legendre functions P~_n^m(x) for n <= nmax (index n(n+1)/2+m).
    void legendre(int nmax, double x, std::vector<double> &P)
    {
      auto tri = [](int n, int m) { return n * (n + 1) / 2 + m; };
      P.assign((nmax + 1) * (nmax + 2) / 2, 0.0);
      double s = std::sqrt(std::max(0.0, 1.0 - x * x));
      P[0]     = 1.0;
      for (int m = 1; m <= nmax; ++m)
        P[tri(m, m)] = -std::sqrt((2.0 * m - 1.0) / (2.0 * m)) * s * P[tri(m - 1, m - 1)];
      for (int m = 0; m < nmax; ++m)
        P[tri(m + 1, m)] = x * std::sqrt(2.0 * m + 1.0) * P[tri(m, m)];
      for (int m = 0; m <= nmax; ++m)
        for (int n = m + 2; n <= nmax; ++n)
          P[tri(n, m)] = ((2.0 * n - 1.0) * x * P[tri(n - 1, m)] -
                          std::sqrt(double((n - 1) * (n - 1) - m * m)) * P[tri(n - 2, m)]) /
                         std::sqrt(double(n * n - m * m));
    }
    inline double Pnm(const std::vector<double> &P, int n, int m)
    {
      return P[n * (n + 1) / 2 + std::abs(m)];
    }

    // mode 0: a = M, 1: a = conj(M), 2: a = Re(M)
    inline void spread(double *T, int K, int nt, int mt, cplx c, int ns, int ms, int mode,
                       double scale)
    {
      c *= scale;
      int sre = ridx(ns, ms, 0), sim = ms ? ridx(ns, ms, 1) : -1;
      int ore = ridx(nt, mt, 0), oim = mt ? ridx(nt, mt, 1) : -1;
      T[size_t(ore) * K + sre] += c.real();
      if (sim >= 0 && mode != 2)
        T[size_t(ore) * K + sim] += mode == 0 ? -c.imag() : c.imag();
      if (oim >= 0)
        {
          T[size_t(oim) * K + sre] += c.imag();
          if (sim >= 0 && mode != 2)
            T[size_t(oim) * K + sim] += mode == 0 ? c.real() : -c.real();
        }
    }
    void sph(const double r[3], double &rho, double &ca, double &be)
    {
      rho = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      ca  = r[2] / rho;
      be  = std::atan2(r[1], r[0]);
    }
  } // namespace

  // child (side 1) -> parent (side 2); rel = child centre - parent centre
  static void m2m_op(int p, const double rel[3], double *T)
  {
    const int K = (p + 1) * (p + 1);
    std::fill(T, T + size_t(K) * K, 0.0);
    double rho, ca, be;
    sph(rel, rho, ca, be);
    std::vector<double> P;
    legendre(p, ca, P);
    const Anm &a = A();
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        for (int nn = 0; nn <= n; ++nn)
          for (int mm = -nn; mm <= nn; ++mm)
            {
              if (std::abs(m - mm) > n - nn)
                continue;
              double rf = Pnm(P, nn, mm) * std::pow(rho, double(nn)) * a(nn, mm) *
                          a(n - nn, m - mm) / a(n, m) *
                          re_ipow(std::abs(m) - std::abs(mm) - std::abs(m - mm));
              cplx c    = rf * std::polar(1.0, -mm * be);
              int  mode = (m - mm) > 0 ? 0 : ((m - mm) < 0 ? 1 : 2);
              spread(T, K, n, m, c, n - nn, std::abs(m - mm), mode, 1.0 / std::pow(2.0, n));
            }
  }

  // parent (side 2) -> child (side 1); rel = parent centre - child centre
  static void l2l_op(int p, const double rel[3], double *T)
  {
    const int K = (p + 1) * (p + 1);
    std::fill(T, T + size_t(K) * K, 0.0);
    double rho, ca, be;
    sph(rel, rho, ca, be);
    std::vector<double> P;
    legendre(p, ca, P);
    const Anm &a = A();
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        for (int nn = n; nn <= p; ++nn)
          for (int mm = -nn; mm <= nn; ++mm)
            {
              if (std::abs(mm - m) > nn - n)
                continue;
              double LC = a(nn - n, mm - m) / a(nn, mm) * a(n, m) *
                          re_ipow(std::abs(mm) - std::abs(mm - m) - std::abs(m)) *
                          std::pow(-1., nn + n);
              double rf   = Pnm(P, nn - n, mm - m) * std::pow(rho, double(nn - n)) * LC;
              cplx   c    = rf * cplx(std::cos((mm - m) * be), std::sin((mm - m) * be));
              int    mode = mm > 0 ? 0 : (mm < 0 ? 1 : 2);
              spread(T, K, n, m, c, nn, std::abs(mm), mode, 1.0 / std::pow(2.0, nn + 1));
            }
  }

  void build_m2l_op(int p, int dx, int dy, int dz, double *T)
  {
    const int K = (p + 1) * (p + 1);
    std::fill(T, T + size_t(K) * K, 0.0);
    double rel[3] = {double(dx), double(dy), double(dz)};
    double rho, ca, be;
    sph(rel, rho, ca, be);
    std::vector<double> P;
    legendre(2 * p, ca, P);
    const Anm &a = A();
    for (int n = 0; n <= p; ++n)
      for (int m = 0; m <= n; ++m)
        for (int nn = 0; nn <= p; ++nn)
          {
            double rhoFact = std::pow(rho, double(-n - nn - 1));
            for (int mm = -nn; mm <= nn; ++mm)
              {
                double C = a(nn, mm) / a(n + nn, m - mm) * a(n, m) *
                           re_ipow(std::abs(m - mm) - std::abs(m) - std::abs(mm)) /
                           std::pow(-1., nn);
                double rf = Pnm(P, nn + n, mm - m) * rhoFact * C;
                cplx   c  = rf * cplx(std::cos((mm - m) * be), std::sin((mm - m) * be));
                spread(T, K, n, m, c, nn, std::abs(mm), mm < 0 ? 1 : 0, 1.0);
              }
          }
  }

  void build_m2m_ops(int p, std::vector<double> &ops)
  {
    const int K = (p + 1) * (p + 1);
    ops.assign(size_t(8) * K * K, 0.0);
    for (int dg = 0; dg < 8; ++dg)
      {
        double rel[3] = {child_off[dg][0] - 0.5, child_off[dg][1] - 0.5, child_off[dg][2] - 0.5};
        m2m_op(p, rel, &ops[size_t(dg) * K * K]);
      }
  }

  void build_l2l_ops(int p, std::vector<double> &ops)
  {
    const int K = (p + 1) * (p + 1);
    ops.assign(size_t(8) * K * K, 0.0);
    for (int dg = 0; dg < 8; ++dg)
      {
        double rel[3] = {0.5 - child_off[dg][0], 0.5 - child_off[dg][1], 0.5 - child_off[dg][2]};
        l2l_op(p, rel, &ops[size_t(dg) * K * K]);
      }
  }

  // ---------------------------------------------------------------------
  // Quadrature rules.
  // ---------------------------------------------------------------------
  static void gauss01(int n, std::vector<double> &x, std::vector<double> &w)
  {
    // Newton iteration on the Legendre polynomial P_n
    std::vector<std::pair<double, double>> xw(n);
    for (int i = 0; i < n; ++i)
      {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it)
          {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j)
              {
                double p3 = p2;
                p2        = p1;
                p1        = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
              }
            pp        = n * (z * p1 - p2) / (z * z - 1.0);
            double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16)
              break;
          }
        double p1 = 1, p2 = 0;
        for (int j = 1; j <= n; ++j)
          {
            double p3 = p2;
            p2        = p1;
            p1        = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
          }
        pp    = n * (z * p1 - p2) / (z * z - 1.0);
        xw[i] = {0.5 * (1.0 - z), 1.0 / ((1.0 - z * z) * pp * pp)};
      }
    std::sort(xw.begin(), xw.end());
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i)
      {
        x[i] = xw[i].first;
        w[i] = xw[i].second;
      }
  }

  // Telles (1987) cubic transformation clustering a Gauss rule at s in {0,1}.
  static void telles01(int n, int s, std::vector<double> &x, std::vector<double> &w)
  {
    std::vector<double> gx, gw;
    gauss01(n, gx, gw);
    const double eb = 2.0 * s - 1.0, es = eb * eb - 1.0;
    const double gb =
      es == 0.0 ? eb : std::cbrt(eb * es + std::fabs(es)) + std::cbrt(eb * es - std::fabs(es)) + eb;
    x.resize(n);
    w.resize(n);
    for (int q = 0; q < n; ++q)
      {
        double g   = 2.0 * gx[q] - 1.0;
        double eta = (std::pow(g - gb, 3.0) + gb * (gb * gb + 3.0)) / (1.0 + 3.0 * gb * gb);
        x[q]       = 0.5 * (eta + 1.0);
        w[q]       = gw[q] * 3.0 * (g - gb) * (g - gb) / (1.0 + 3.0 * gb * gb);
      }
  }

  static void tensor(const std::vector<double> &x1, const std::vector<double> &w1,
                     const std::vector<double> &x2, const std::vector<double> &w2,
                     std::vector<double> &pts, std::vector<double> &w)
  {
    pts.clear();
    w.clear();
    for (size_t j = 0; j < x2.size(); ++j)
      for (size_t i = 0; i < x1.size(); ++i)
        {
          pts.push_back(x1[i]);
          pts.push_back(x2[j]);
          w.push_back(w1[i] * w2[j]);
        }
  }

  void gauss_rule_2d(int n, std::vector<double> &pts, std::vector<double> &w)
  {
    std::vector<double> x, wx;
    gauss01(n, x, wx);
    tensor(x, wx, x, wx, pts, w);
  }

  void telles_rule_2d(int n, int vertex, std::vector<double> &pts, std::vector<double> &w)
  {
    std::vector<double> x1, w1, x2, w2;
    telles01(n, vertex & 1, x1, w1);
    telles01(n, (vertex >> 1) & 1, x2, w2);
    tensor(x1, w1, x2, w2, pts, w);
  }
} // namespace pibem

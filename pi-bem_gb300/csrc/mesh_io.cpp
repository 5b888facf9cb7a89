// Mesh ingestion on the host: UCD (.inp) surface meshes, double-node sets and
// Dirichlet masks from material ids -- the inputs pi-BEM builds before it calls
// the operator:
//   ComputationalDomain::read_domain (source/computational_domain.cc:258-300),
//     GridIn::read_ucd for "inp" files (:286-287);
//   the double-node sets of coincident support points that BEMProblem hands to
//     BEMFMA::init_fma (source/bem_problem.cc:200);
//   BEMProblem::compute_dirichlet_and_neumann_dofs_vectors
//     (source/bem_problem.cc:315-411): a DoF is Dirichlet when any cell it
//     belongs to carries one of the Dirichlet material ids.
// Plain C ABI (pibem_gpu.h); no device code, no GPU needed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pibem_gpu.h"

namespace
{
  struct UcdMesh
  {
    std::vector<double>  xyz;
    std::vector<int32_t> cells, material;
  };

  // AVS UCD ASCII: "n_nodes n_cells n_node_data n_cell_data n_model_data",
  // n_nodes lines "id x y z", n_cells lines "id material type v...".  Only
  // "quad" cells are surface cells of a Q1 BEM mesh; their vertices are listed
  // counterclockwise (seen from the side the normal points to) and are stored
  // here in deal.II's lexicographic order (v0, v1, v3, v2).  Lines starting
  // with '#' are comments.
  int read_ucd(const char *path, UcdMesh &m, std::string &err)
  {
    std::ifstream in(path);
    if (!in)
      {
        err = "cannot open file";
        return PIBEM_EINVAL;
      }
    std::string line;
    auto        next = [&](std::string &l) {
      while (std::getline(in, l))
        if (!l.empty() && l[0] != '#' && l.find_first_not_of(" \t\r") != std::string::npos)
          return true;
      return false;
    };
    if (!next(line))
      {
        err = "empty file";
        return PIBEM_EINVAL;
      }
    long long nn = -1, nc = -1;
    {
      std::istringstream h(line);
      if (!(h >> nn >> nc) || nn < 0 || nc < 0)
        {
          err = "bad header";
          return PIBEM_EINVAL;
        }
    }
    std::unordered_map<long long, int32_t> id_of;
    m.xyz.resize(size_t(3 * nn));
    for (long long i = 0; i < nn; ++i)
      {
        long long id;
        double    x, y, z;
        if (!next(line))
          {
            err = "missing node lines";
            return PIBEM_EINVAL;
          }
        std::istringstream l(line);
        if (!(l >> id >> x >> y >> z))
          {
            err = "bad node line: " + line;
            return PIBEM_EINVAL;
          }
        if (!id_of.emplace(id, int32_t(i)).second)
          {
            err = "duplicate node id " + std::to_string(id);
            return PIBEM_EINVAL;
          }
        m.xyz[3 * i] = x, m.xyz[3 * i + 1] = y, m.xyz[3 * i + 2] = z;
      }
    m.cells.clear();
    m.material.clear();
    for (long long c = 0; c < nc; ++c)
      {
        if (!next(line))
          {
            err = "missing cell lines";
            return PIBEM_EINVAL;
          }
        std::istringstream l(line);
        long long          id, mat;
        std::string        type;
        if (!(l >> id >> mat >> type))
          {
            err = "bad cell line: " + line;
            return PIBEM_EINVAL;
          }
        if (type != "quad")
          continue; // lines / points (boundary indicators of a surface mesh)
        long long v[4];
        for (auto &x : v)
          if (!(l >> x))
            {
              err = "bad quad line: " + line;
              return PIBEM_EINVAL;
            }
        int32_t q[4];
        for (int k = 0; k < 4; ++k)
          {
            auto f = id_of.find(v[k]);
            if (f == id_of.end())
              {
                err = "quad refers to unknown node " + std::to_string(v[k]);
                return PIBEM_EINVAL;
              }
            q[k] = f->second;
          }
        m.cells.insert(m.cells.end(), {q[0], q[1], q[3], q[2]});
        m.material.push_back(int32_t(mat));
      }
    return PIBEM_OK;
  }

  thread_local std::string t_err;
} // namespace

extern "C"
{
  int pibem_ucd_read(const char *path, int64_t *n_nodes, int64_t *n_cells, double *xyz,
                     int32_t *cell_nodes, int32_t *material_id)
  {
    if (!path || !n_nodes || !n_cells)
      return PIBEM_EINVAL;
    UcdMesh m;
    int     rc = read_ucd(path, m, t_err);
    if (rc != PIBEM_OK)
      return rc;
    const int64_t nn = int64_t(m.xyz.size() / 3), nc = int64_t(m.material.size());
    if (xyz || cell_nodes || material_id)
      {
        if (!xyz || !cell_nodes || *n_nodes < nn || *n_cells < nc)
          {
            t_err = "output arrays missing or too small";
            return PIBEM_EINVAL;
          }
        std::copy(m.xyz.begin(), m.xyz.end(), xyz);
        std::copy(m.cells.begin(), m.cells.end(), cell_nodes);
        if (material_id)
          std::copy(m.material.begin(), m.material.end(), material_id);
      }
    *n_nodes = nn;
    *n_cells = nc;
    return PIBEM_OK;
  }

  const char *pibem_mesh_io_error(void) { return t_err.c_str(); }

  int pibem_double_nodes(int64_t n_nodes, const double *xyz, double tol, int32_t *offsets,
                         int32_t *ids, int64_t capacity, int64_t *n_ids)
  {
    if (n_nodes < 0 || (n_nodes > 0 && !xyz) || !offsets || !n_ids || !(tol >= 0))
      return PIBEM_EINVAL;
    // sort by x, sweep a window of width tol; groups are the connected sets
    // of nodes closer than tol in every coordinate (union-find)
    std::vector<int64_t> order(static_cast<size_t>(n_nodes)), parent(static_cast<size_t>(n_nodes));
    std::iota(order.begin(), order.end(), 0);
    std::iota(parent.begin(), parent.end(), 0);
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
      return xyz[3 * a] < xyz[3 * b] || (xyz[3 * a] == xyz[3 * b] && a < b);
    });
    auto find = [&](int64_t a) {
      while (parent[a] != a)
        a = parent[a] = parent[parent[a]];
      return a;
    };
    for (int64_t i = 0; i < n_nodes; ++i)
      for (int64_t j = i + 1; j < n_nodes && xyz[3 * order[j]] - xyz[3 * order[i]] <= tol; ++j)
        {
          const int64_t a = order[i], b = order[j];
          if (std::fabs(xyz[3 * a + 1] - xyz[3 * b + 1]) <= tol &&
              std::fabs(xyz[3 * a + 2] - xyz[3 * b + 2]) <= tol)
            {
              int64_t ra = find(a), rb = find(b);
              if (ra != rb)
                parent[std::max(ra, rb)] = std::min(ra, rb);
            }
        }
    // every node's set lists all members of its group (itself included), in
    // increasing order
    std::vector<std::vector<int32_t>> members(static_cast<size_t>(n_nodes));
    for (int64_t i = 0; i < n_nodes; ++i)
      members[size_t(find(i))].push_back(int32_t(i));
    int64_t total = 0;
    offsets[0]    = 0;
    for (int64_t i = 0; i < n_nodes; ++i)
      {
        const auto &g = members[size_t(find(i))];
        if (ids && total + int64_t(g.size()) <= capacity)
          std::copy(g.begin(), g.end(), ids + total);
        total += int64_t(g.size());
        offsets[i + 1] = int32_t(total);
      }
    *n_ids = total;
    return ids && total > capacity ? PIBEM_EINVAL : PIBEM_OK;
  }

  int pibem_dirichlet_mask_from_materials(int64_t n_nodes, int64_t n_cells,
                                          const int32_t *cell_nodes, const int32_t *material_id,
                                          int32_t n_dirichlet_ids, const int32_t *dirichlet_ids,
                                          uint8_t *mask)
  {
    if (n_nodes < 0 || n_cells < 0 || !mask || (n_cells > 0 && (!cell_nodes || !material_id)) ||
        n_dirichlet_ids < 0 || (n_dirichlet_ids > 0 && !dirichlet_ids))
      return PIBEM_EINVAL;
    std::fill(mask, mask + n_nodes, uint8_t(0));
    for (int64_t c = 0; c < n_cells; ++c)
      if (std::find(dirichlet_ids, dirichlet_ids + n_dirichlet_ids, material_id[c]) !=
          dirichlet_ids + n_dirichlet_ids)
        for (int k = 0; k < 4; ++k)
          {
            const int32_t v = cell_nodes[4 * c + k];
            if (v < 0 || v >= n_nodes)
              return PIBEM_EINVAL;
            mask[v] = 1;
          }
    return PIBEM_OK;
  }
}

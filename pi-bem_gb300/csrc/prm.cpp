// Parameters: the reference's defaults and a reader for the knobs of a deal.II
// parameter file (subsection / set / end), so that an existing pi-BEM .prm
// configures this library unchanged:
//   BEMFMA<3>/FMA Params/FMA Truncation Order                 (bem_fma.cc:76-80)
//   BEMFMA<3>/Octree Params/Number of Octree Levels,
//     Maximum Number of Collocation Points per Childless Block (bem_fma.cc:67-74)
//   BEMProblem<3>/Quadrature rules/Quadrature order, Singular quadrature order
//   BEMProblem<3>/Solver/Max steps, Tolerance                 (bem_problem.cc:255-256)
//   BEMProblem<3>/Is external flow                            (bem_problem.cc:281)
// New knobs live in the added subsection "GB300 Params".
#include <cctype>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/pibem_gpu.h"

namespace
{
  std::string trim(const std::string &s)
  {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a]))
      ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1]))
      --b;
    return s.substr(a, b - a);
  }
  bool as_bool(const std::string &v)
  {
    std::string t;
    for (char c : v)
      t += char(std::tolower((unsigned char)c));
    return t == "true" || t == "1" || t == "yes" || t == "on";
  }
} // namespace

extern "C" int pibem_params_default(pibem_params *p)
{
  if (!p)
    return PIBEM_EINVAL;
  p->fma_truncation_order          = 6;
  p->num_octree_levels             = 10;
  p->max_nodes_per_childless_block = 20;
  p->quadrature_order              = 4;
  p->singular_quadrature_order     = 5;
  p->solver_max_steps              = 3000;
  p->solver_tolerance              = 1e-8;
  p->gmres_restart                 = 100;
  p->is_external_flow              = 0;
  p->precision_mode                = PIBEM_PRECISION_FP64;
  p->preconditioner                = 1;
  p->device                        = 0;
  p->inner_tolerance               = 1e-4;
  p->hbm_budget_gb                 = 0.0;
  p->m2l_engine                    = PIBEM_M2L_TENSOR_CORE;
  p->double_body                   = 0;
  p->symmetry_plane_z_level        = 0.0;
  p->continuous_gradient           = 1;
  p->m2l_chunk_pairs               = 0;
  p->m2l_stages                    = 0;
  return PIBEM_OK;
}

extern "C" int pibem_params_from_prm(pibem_params *p, const char *text)
{
  if (!p || !text)
    return PIBEM_EINVAL;
  std::istringstream       in(text);
  std::string              line;
  std::vector<std::string> stack;
  while (std::getline(in, line))
    {
      size_t hash = line.find('#');
      if (hash != std::string::npos)
        line = line.substr(0, hash);
      line = trim(line);
      if (line.empty())
        continue;
      if (line.rfind("subsection", 0) == 0)
        {
          stack.push_back(trim(line.substr(10)));
          continue;
        }
      if (line == "end")
        {
          if (!stack.empty())
            stack.pop_back();
          continue;
        }
      if (line.rfind("set", 0) != 0)
        continue;
      size_t eq = line.find('=');
      if (eq == std::string::npos)
        continue;
      std::string key = trim(line.substr(3, eq - 3));
      std::string val = trim(line.substr(eq + 1));
      std::string sec = stack.empty() ? "" : stack.back();
      std::string top = stack.empty() ? "" : stack.front();
      const char *v   = val.c_str();
      if (sec == "FMA Params" && key == "FMA Truncation Order")
        p->fma_truncation_order = std::atoi(v);
      else if (sec == "Octree Params" && key == "Number of Octree Levels")
        p->num_octree_levels = std::atoi(v);
      else if (sec == "Octree Params" &&
               key == "Maximum Number of Collocation Points per Childless Block")
        p->max_nodes_per_childless_block = std::atoi(v);
      else if (sec == "Quadrature rules" && key == "Quadrature order")
        p->quadrature_order = std::atoi(v);
      else if (sec == "Quadrature rules" && key == "Singular quadrature order")
        p->singular_quadrature_order = std::atoi(v);
      else if (sec == "Solver" && top == "BEMProblem<3>" && key == "Max steps")
        p->solver_max_steps = std::atoi(v);
      else if (sec == "Solver" && top == "BEMProblem<3>" && key == "Tolerance")
        p->solver_tolerance = std::atof(v);
      else if (sec == "BEMProblem<3>" && key == "Is external flow")
        p->is_external_flow = as_bool(val) ? 1 : 0;
      else if (sec == "BEMProblem<3>" && key == "Symmetry plane z level")
        p->symmetry_plane_z_level = std::atof(v);
      else if (sec == "BEMProblem<3>" && key == "Continuos gradient across edges")
        p->continuous_gradient = as_bool(val) ? 1 : 0;
      else if (sec == "GB300 Params")
        {
          if (key == "Precision mode")
            p->precision_mode = (val == "Mixed" || val == "mixed" || val == "1")
                                  ? PIBEM_PRECISION_MIXED
                                  : (val == "FloatFloat" || val == "float-float" || val == "2")
                                      ? PIBEM_PRECISION_FLOAT_FLOAT
                                      : PIBEM_PRECISION_FP64;
          else if (key == "Preconditioner")
            p->preconditioner = (val == "none" || val == "None" || val == "0")  ? 0
                                : (val == "ILU" || val == "ilu" || val == "2") ? 2
                                                                              : 1;
          else if (key == "GMRES restart")
            p->gmres_restart = std::atoi(v);
          else if (key == "Inner tolerance")
            p->inner_tolerance = std::atof(v);
          else if (key == "HBM budget GB")
            p->hbm_budget_gb = std::atof(v);
          else if (key == "Device")
            p->device = std::atoi(v);
          else if (key == "Double body")
            p->double_body = as_bool(val) ? 1 : 0;
          else if (key == "M2L engine")
            p->m2l_engine = (val == "CUDA cores" || val == "cuda" || val == "1")
                              ? PIBEM_M2L_CUDA_CORE
                              : PIBEM_M2L_TENSOR_CORE;
          else if (key == "M2L chunk pairs")
            p->m2l_chunk_pairs = std::atoi(v);
          else if (key == "M2L stages")
            p->m2l_stages = std::atoi(v);
        }
    }
  return PIBEM_OK;
}

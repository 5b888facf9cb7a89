// Test harness: exposes the host octree builder (pi-bem_gb300/csrc/tree.cpp) to
// ctypes so that its boxes and lists can be compared with the oracle on the CPU.
#include "../../pi-bem_gb300/csrc/pibem_internal.h"
#include <algorithm>
using namespace pibem;
static Tree T; static MeshHost M;
extern "C" int th_build(int n, const double* xyz, int nc, const int* cells, const double* qpts, int nq, int L, int maxn) {
  M.n_nodes=n; M.n_cells=nc; M.n_dofs=n; M.n_cells_body=nc; M.xyz.assign(xyz,xyz+3*n); M.cells.assign(cells,cells+4*nc);
  M.dbl_off.resize(n+1); M.dbl_ids.resize(n); for(int i=0;i<=n;i++) M.dbl_off[i]=i; for(int i=0;i<n;i++) M.dbl_ids[i]=i;
  M.elem_off.assign(n+1,0); for(int i=0;i<4*nc;i++) M.elem_off[cells[i]+1]++; for(int i=0;i<n;i++) M.elem_off[i+1]+=M.elem_off[i];
  M.elem_ids.assign(M.elem_off[n],0); std::vector<int> f(M.elem_off.begin(),M.elem_off.end()-1); for(int c=0;c<nc;c++) for(int j=0;j<4;j++) M.elem_ids[f[cells[4*c+j]]++]=c;
  std::vector<double> q(qpts, qpts+3*(size_t)nc*nq);
  build_tree(M,q,nq,L,maxn,T); return T.nb; }
extern "C" void th_boxes(int* level,int* parent,int* nchild,double* pmin,double* delta,int* nn,int* nqq){
  for(int b=0;b<T.nb;b++){level[b]=T.level[b];parent[b]=T.parent[b];nchild[b]=T.nchild[b];for(int k=0;k<3;k++)pmin[3*b+k]=T.pmin[3*b+k];delta[b]=T.delta[b];nn[b]=T.nend[b]-T.nbeg[b];nqq[b]=T.qend[b]-T.qbeg[b];}}
extern "C" int th_list(int kind,int b,int sub,int* out,int cap){auto&L=kind==0?T.nn[b]:kind==1?T.il[b]:T.nil[b]; if(sub>=(int)L.size()) return -1; for(int i=0;i<(int)L[sub].size()&&i<cap;i++) out[i]=L[sub][i]; return L[sub].size();}
extern "C" int th_nsub(int b){return T.nn[b].size();}
extern "C" int th_childless(int* out){for(size_t i=0;i<T.childless.size();i++) out[i]=T.childless[i]; return T.childless.size();}

// Double body: mirror_mesh + octree + plan of the mirrored geometry; reports
// what the plan's kernels would index.  st: [near rows, max row node, max column,
// max P2M dof, L2P nodes, M2L pairs, M2L targets without collocation nodes,
// M2P pairs, M2P targets without collocation nodes, rows that are not
// distinct, L2L boxes without collocation nodes]
extern "C" int th_plan_mirrored(int n, const double* xyz, int nc, const int* cells, double z0,
                                const double* qpts, int nq, int L, int maxn, int p, long* st) {
  std::vector<std::vector<int32_t>> sets(n); for(int i=0;i<n;i++) sets[i]={i};
  MeshHost m; mirror_mesh(n, xyz, nc, cells, sets, true, z0, m);
  m.elem_off.assign(m.n_nodes+1,0); for(size_t i=0;i<m.cells.size();i++) m.elem_off[m.cells[i]+1]++;
  for(int64_t i=0;i<m.n_nodes;i++) m.elem_off[i+1]+=m.elem_off[i];
  m.elem_ids.assign(m.elem_off[m.n_nodes],0); std::vector<int> f(m.elem_off.begin(),m.elem_off.end()-1);
  for(int64_t c=0;c<m.n_cells;c++) for(int j=0;j<4;j++) m.elem_ids[f[m.cells[4*c+j]]++]=int(c);
  std::vector<double> q(qpts, qpts+3*(size_t)m.n_cells*nq);
  Tree t; build_tree(m,q,nq,L,maxn,t); Plan pl; build_plan(m,t,nq,p,pl);
  auto has_real=[&](int b){for(int k=t.nbeg[b];k<t.nend[b];k++) if(t.node_sorted[k]<n) return true; return false;};
  for(int i=0;i<11;i++) st[i]=0;
  st[0]=pl.nrows.size(); for(int v:pl.nrows) st[1]=std::max<long>(st[1],v);
  for(int v:pl.ncols) st[2]=std::max<long>(st[2],v); for(int v:pl.prow_dof) st[3]=std::max<long>(st[3],v);
  st[4]=pl.lnode_ids.size(); st[5]=pl.n_m2l; for(int b:pl.m2l_tgt) st[6]+=!has_real(b);
  st[7]=pl.n_m2p; for(int b:pl.m2p_tgt) st[8]+=!has_real(b);
  std::vector<int> r(pl.nrows.begin(),pl.nrows.end()); std::sort(r.begin(),r.end());
  st[9]=long(r.size())-long(std::unique(r.begin(),r.end())-r.begin());
  for(int b:pl.l2l_box) st[10]+=!has_real(b);
  return t.nb; }

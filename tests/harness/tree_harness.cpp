// Test harness: exposes the host octree builder (pi-bem_gb300/csrc/tree.cpp) to
// ctypes so that its boxes and lists can be compared with the oracle on the CPU.
#include "../../pi-bem_gb300/csrc/pibem_internal.h"
#include <algorithm>
using namespace pibem;
static Tree T; static MeshHost M;
extern "C" int th_build(int n, const double* xyz, int nc, const int* cells, const double* qpts, int nq, int L, int maxn) {
  M.n_nodes=n; M.n_cells=nc; M.xyz.assign(xyz,xyz+3*n); M.cells.assign(cells,cells+4*nc);
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

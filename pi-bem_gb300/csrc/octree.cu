// The octree and the three interaction lists of pi-BEM's
// BEMFMA::generate_octree_blocking (source/bem_fma.cc:3615-4801), built on the
// device.  The box set, the box numbering and every list are those of the host
// builder in tree.cpp (same rules, same floating-point comparisons):
//   * path keys of the nodes and quadrature points by the reference's own
//     comparisons (bem_fma.cc:3844-3973), one thread per point;
//   * a stable LSD radix sort of (key, id), 8 bits a pass;
//   * per level the boxes are the distinct key prefixes of the points not yet
//     in a childless box, in ascending prefix order (the reference's
//     breadth-first numbering: parents in order, children by digit); their node
//     and quadrature ranges by binary search; the childless test on the host
//     from the node counts (weights 1 / |double set|);
//   * near neighbours (TOLL touch test), intList (near neighbours plus the
//     boxes of the quadrature points of the cells around a box's nodes and
//     their doubles) and nonIntList, one block per box and level, each list
//     gathered into a bitmap of box ids in shared memory and read out in
//     ascending order.
// A tree whose box-id bitmap or lists exceed the builder's capacities (an
// unusual mesh) is reported, and the caller builds the tree on the host.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iterator>
#include <vector>

#include "kernels.h"
#include "pibem_internal.h"

namespace pibem
{
  namespace
  {
    constexpr double OT_TOLL = 0.001; // source/bem_fma.cc:1
    __constant__ int c_digit_of[2][2][2] = {{{0, 1}, {3, 2}}, {{4, 5}, {7, 6}}}; // [hz][hy][hx]

    inline unsigned nblk(int64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

    // max |x| over the coordinates (non-negative doubles order as their bits)
    __global__ void absmax_kernel(int64_t n, const double *__restrict__ x,
                                  unsigned long long *__restrict__ out)
    {
      double m = 0;
      for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
           i += int64_t(gridDim.x) * blockDim.x)
        m = fmax(m, fabs(x[i]));
      for (int o = 16; o > 0; o >>= 1)
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if ((threadIdx.x & 31) == 0)
        atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
    }

    // path key of every point with the reference's comparisons (a point on a
    // split plane goes to the low side)
    __global__ void keys_kernel(int64_t n, const double *__restrict__ pts, double p0, double delta0,
                                int L, uint64_t *__restrict__ key, int32_t *__restrict__ id)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n)
        return;
      const double x0 = pts[3 * i], x1 = pts[3 * i + 1], x2 = pts[3 * i + 2];
      double       pm0 = p0, pm1 = p0, pm2 = p0, d = delta0;
      uint64_t     k   = 0;
      for (int l = 1; l <= L; ++l)
        {
          d /= 2.;
          const bool hx = !(x0 <= pm0 + d);
          const bool hy = !(x1 <= pm1 + d);
          const bool hz = !(x2 <= pm2 + d);
          k             = (k << 3) | uint64_t(c_digit_of[hz][hy][hx]);
          if (hx)
            pm0 = pm0 + d;
          if (hy)
            pm1 = pm1 + d;
          if (hz)
            pm2 = pm2 + d;
        }
      key[i] = k;
      id[i]  = int32_t(i);
    }

    // ---- stable LSD radix sort of (key, value), 8 bits a pass ---------------
    constexpr int RS_THREADS = 256, RS_ROUNDS = 8, RS_TILE = RS_THREADS * RS_ROUNDS;

    __global__ void __launch_bounds__(RS_THREADS)
      rs_hist_kernel(int64_t n, const uint64_t *__restrict__ key, int shift, int ntiles,
                     uint32_t *__restrict__ counts)
    {
      __shared__ uint32_t h[256];
      h[threadIdx.x] = 0;
      __syncthreads();
      for (int r = 0; r < RS_ROUNDS; ++r)
        {
          const int64_t i = int64_t(blockIdx.x) * RS_TILE + r * RS_THREADS + threadIdx.x;
          if (i < n)
            atomicAdd(&h[(key[i] >> shift) & 255u], 1u);
        }
      __syncthreads();
      counts[int64_t(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
    }

    // exclusive scan of m values in place, one block of 1024 threads
    __global__ void __launch_bounds__(1024) scan_kernel(int64_t m, uint32_t *__restrict__ v,
                                                        uint32_t *__restrict__ total)
    {
      __shared__ uint32_t part[1024];
      const int64_t seg = (m + 1023) / 1024;
      const int64_t a = int64_t(threadIdx.x) * seg, b = min(m, a + seg);
      uint32_t      s = 0;
      for (int64_t i = a; i < b; ++i)
        s += v[i];
      part[threadIdx.x] = s;
      __syncthreads();
      for (int o = 1; o < 1024; o <<= 1)
        {
          const uint32_t add = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
          __syncthreads();
          part[threadIdx.x] += add;
          __syncthreads();
        }
      uint32_t run = part[threadIdx.x] - s; // exclusive
      for (int64_t i = a; i < b; ++i)
        {
          const uint32_t x = v[i];
          v[i]             = run;
          run += x;
        }
      if (total && threadIdx.x == 1023)
        *total = part[1023];
    }

    // each tile's items in index order: the rank of an item among the items of
    // its digit before it, from per-warp matches and per-digit running counts
    __global__ void __launch_bounds__(RS_THREADS)
      rs_scatter_kernel(int64_t n, const uint64_t *__restrict__ kin, const int32_t *__restrict__ vin,
                        uint64_t *__restrict__ kout, int32_t *__restrict__ vout, int shift,
                        int ntiles, const uint32_t *__restrict__ offs)
    {
      __shared__ uint32_t run[256];
      __shared__ uint32_t wc[RS_THREADS / 32][256];
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      run[threadIdx.x] = 0;
      for (int r = 0; r < RS_ROUNDS; ++r)
        {
          for (int w = 0; w < RS_THREADS / 32; ++w)
            wc[w][threadIdx.x] = 0;
          __syncthreads();
          const int64_t  i     = int64_t(blockIdx.x) * RS_TILE + r * RS_THREADS + threadIdx.x;
          const bool     valid = i < n;
          const unsigned mask  = __ballot_sync(0xffffffffu, valid);
          uint64_t       k     = 0;
          int            d = 0, rank = 0;
          if (valid)
            {
              k                    = kin[i];
              d                    = int((k >> shift) & 255u);
              const unsigned peers = __match_any_sync(mask, d);
              rank                 = __popc(peers & ((1u << lane) - 1u));
              if (rank == 0)
                wc[warp][d] = __popc(peers);
            }
          __syncthreads();
          {
            uint32_t acc = run[threadIdx.x];
            for (int w = 0; w < RS_THREADS / 32; ++w)
              {
                const uint32_t c     = wc[w][threadIdx.x];
                wc[w][threadIdx.x]   = acc;
                acc += c;
              }
            run[threadIdx.x] = acc;
          }
          __syncthreads();
          if (valid)
            {
              const uint32_t pos = offs[int64_t(d) * ntiles + blockIdx.x] + wc[warp][d] + uint32_t(rank);
              kout[pos]          = k;
              vout[pos]          = vin[i];
            }
          __syncthreads();
        }
    }

    // ---- levels -------------------------------------------------------------
    // flag[i] = 1 where a run of equal prefixes starts among the active points
    __global__ void run_start_kernel(int64_t n, const uint64_t *__restrict__ key,
                                     const uint8_t *__restrict__ act, int shift,
                                     uint32_t *__restrict__ flag)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n)
        return;
      flag[i] = act[i] && (i == 0 || !act[i - 1] || (key[i - 1] >> shift) != (key[i] >> shift));
    }

    // the prefixes of the run starts, compacted (pos: exclusive scan of flag)
    __global__ void run_compact_kernel(int64_t n, const uint64_t *__restrict__ key,
                                       const uint8_t *__restrict__ act, int shift,
                                       const uint32_t *__restrict__ pos, uint64_t *__restrict__ out)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n)
        return;
      if (act[i] && (i == 0 || !act[i - 1] || (key[i - 1] >> shift) != (key[i] >> shift)))
        out[pos[i]] = key[i] >> shift;
    }

    // [lower_bound(P << shift), lower_bound((P + 1) << shift)) of each box prefix
    __global__ void box_range_kernel(int nbx, const uint64_t *__restrict__ pfx, int shift, int64_t n,
                                     const uint64_t *__restrict__ key, int32_t *__restrict__ beg,
                                     int32_t *__restrict__ end)
    {
      const int b = blockIdx.x * blockDim.x + threadIdx.x;
      if (b >= nbx)
        return;
      auto lb = [&](uint64_t v) {
        int64_t lo = 0, hi = n;
        while (lo < hi)
          {
            const int64_t mid = (lo + hi) >> 1;
            if (key[mid] < v)
              lo = mid + 1;
            else
              hi = mid;
          }
        return int32_t(lo);
      };
      beg[b] = lb(pfx[b] << shift);
      end[b] = lb((pfx[b] + 1) << shift);
    }

    // the level's box of every active point (binary search of its prefix);
    // points of a childless box leave the active set
    __global__ void assign_kernel(int64_t n, const uint64_t *__restrict__ key, uint8_t *__restrict__ act,
                                  int shift, int nbx, const uint64_t *__restrict__ pfx, int box0,
                                  const uint8_t *__restrict__ childless, int32_t *__restrict__ cur)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n || !act[i])
        return;
      const uint64_t p  = key[i] >> shift;
      int            lo = 0, hi = nbx - 1;
      while (lo < hi)
        {
          const int mid = (lo + hi) >> 1;
          if (pfx[mid] < p)
            lo = mid + 1;
          else
            hi = mid;
        }
      cur[i] = box0 + lo;
      if (childless[lo])
        act[i] = 0;
    }

    // qbox[l][id] = the current box of each (sorted) quadrature point
    __global__ void qbox_kernel(int64_t n, const int32_t *__restrict__ qid, const int32_t *__restrict__ cur,
                                int32_t *__restrict__ qbox_l)
    {
      const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i < n)
        qbox_l[qid[i]] = cur[i];
    }

    // ---- lists -----------------------------------------------------------------
    struct BoxDev
    {
      const double  *pmin, *delta;
      const int32_t *nchild, *child_first, *parent, *nbeg, *nend;
    };

    __device__ inline bool touches(const BoxDev &B, int a, int b)
    {
      double PMin1[3], PMax1[3], PMin2[3], PMax2[3];
      for (int k = 0; k < 3; ++k)
        {
          PMin1[k] = B.pmin[3 * a + k];
          PMax1[k] = 2. * (B.delta[a] / 2.) + PMin1[k];
          PMin2[k] = B.pmin[3 * b + k];
          PMax2[k] = 2. * (B.delta[b] / 2.) + PMin2[k];
        }
      for (int ax = 0; ax < 3; ++ax)
        {
          const int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
          if ((fabs(PMin1[ax] - PMax2[ax]) <= OT_TOLL) || (fabs(PMax1[ax] - PMin2[ax]) <= OT_TOLL))
            if ((PMin1[o1] - OT_TOLL <= PMax2[o1]) && (PMax1[o1] + OT_TOLL >= PMin2[o1]))
              if ((PMin1[o2] - OT_TOLL <= PMax2[o2]) && (PMax1[o2] + OT_TOLL >= PMin2[o2]))
                return true;
        }
      return false;
    }

    // Lists in a flat store: list li = (box, sub) holds cnt[li] ids at
    // store + li * cap.  li = lbase[box] + sub.
    struct ListStore
    {
      int32_t *ids;
      int32_t *cnt;
      int      cap;
    };

    constexpr int OT_THREADS = 256;

    // A set of box ids as a bitmap in shared memory (nwords 32-bit words):
    // insertion by atomicOr, extraction in ascending order (sorted, unique)
    __device__ inline void bm_clear(uint32_t *bm, int nwords)
    {
      for (int w = threadIdx.x; w < nwords; w += blockDim.x)
        bm[w] = 0;
    }
    __device__ inline void bm_add(uint32_t *bm, int v) { atomicOr(&bm[v >> 5], 1u << (v & 31)); }
    __device__ inline bool bm_has(const uint32_t *bm, int v) { return (bm[v >> 5] >> (v & 31)) & 1u; }

    // writes the ids of bm in ascending order into list li of L (count into
    // L.cnt[li]; more than L.cap: error)
    __device__ void bm_extract(const uint32_t *bm, int nwords, const ListStore &L, int li, int *err)
    {
      __shared__ int part[OT_THREADS + 1];
      const int      per = (nwords + blockDim.x - 1) / blockDim.x;
      const int      w0 = threadIdx.x * per, w1 = min(nwords, w0 + per);
      int            c  = 0;
      for (int w = w0; w < w1; ++w)
        c += __popc(bm[w]);
      part[threadIdx.x + 1] = c;
      if (threadIdx.x == 0)
        part[0] = 0;
      __syncthreads();
      if (threadIdx.x == 0)
        for (int t = 1; t <= int(blockDim.x); ++t)
          part[t] += part[t - 1];
      __syncthreads();
      const int total = part[blockDim.x];
      if (total > L.cap)
        {
          if (threadIdx.x == 0)
            atomicExch(err, 1);
        }
      else
        {
          int o = part[threadIdx.x];
          for (int w = w0; w < w1; ++w)
            {
              uint32_t x = bm[w];
              while (x)
                {
                  const int bit = __ffs(x) - 1;
                  x &= x - 1;
                  L.ids[int64_t(li) * L.cap + o++] = w * 32 + bit;
                }
            }
        }
      if (threadIdx.x == 0)
        L.cnt[li] = total > L.cap ? 0 : total;
      __syncthreads();
    }

    // near neighbours of the boxes of one level (bem_fma.cc:4269-4580)
    __global__ void __launch_bounds__(OT_THREADS)
      nn_kernel(int box0, int nbx, int L, int level, int nwords, BoxDev B,
                const int32_t *__restrict__ lbase, ListStore NN, int *err)
    {
      extern __shared__ uint32_t bm[];
      const int b = box0 + blockIdx.x;
      if (blockIdx.x >= nbx)
        return;
      const int ns = B.nchild[b] == 0 ? L - level + 1 : 1;
      for (int sub = 0; sub < ns; ++sub)
        {
          bm_clear(bm, nwords);
          __syncthreads();
          // source list: the parent's sublevel-0 list, or this box's previous sublevel
          const int src = sub == 0 ? lbase[B.parent[b]] : lbase[b] + sub - 1;
          const int cn  = NN.cnt[src];
          if (sub == 0 && threadIdx.x == 0)
            bm_add(bm, b);
          for (int e = threadIdx.x; e < cn; e += blockDim.x)
            {
              const int pos = NN.ids[int64_t(src) * NN.cap + e];
              if (B.nchild[pos] == 0 && (sub > 0 || touches(B, b, pos)))
                bm_add(bm, pos);
              for (int c = 0; c < B.nchild[pos]; ++c)
                if (touches(B, b, B.child_first[pos] + c))
                  bm_add(bm, B.child_first[pos] + c);
            }
          __syncthreads();
          bm_extract(bm, nwords, NN, lbase[b] + sub, err);
        }
    }

    // intList (bem_fma.cc:4612-4668): the near neighbours and the boxes, at the
    // list's level, of the quadrature points of the cells around the box's nodes
    // and their doubles
    __global__ void __launch_bounds__(OT_THREADS)
      il_kernel(int box0, int nbx, int L, int level, int nwords, BoxDev B,
                const int32_t *__restrict__ lbase, const int32_t *__restrict__ node_sorted,
                const int32_t *__restrict__ dbl_off, const int32_t *__restrict__ dbl_ids,
                const int32_t *__restrict__ elem_off, const int32_t *__restrict__ elem_ids, int nq,
                int64_t Q, const int32_t *__restrict__ qbox, ListStore NN, ListStore IL, int *err)
    {
      extern __shared__ uint32_t bm[];
      const int b = box0 + blockIdx.x;
      if (blockIdx.x >= nbx)
        return;
      const int ns = B.nchild[b] == 0 ? L - level + 1 : 1;
      for (int sub = 0; sub < ns; ++sub)
        {
          bm_clear(bm, nwords);
          __syncthreads();
          const int li = lbase[b] + sub;
          const int cn = NN.cnt[li];
          for (int e = threadIdx.x; e < cn; e += blockDim.x)
            bm_add(bm, NN.ids[int64_t(li) * NN.cap + e]);
          const int32_t *qb = qbox + int64_t(level + sub) * Q;
          for (int k = B.nbeg[b] + int(threadIdx.x); k < B.nend[b]; k += blockDim.x)
            {
              const int node = node_sorted[k];
              for (int a = dbl_off[node]; a < dbl_off[node + 1]; ++a)
                {
                  const int dn = dbl_ids[a];
                  for (int e = elem_off[dn]; e < elem_off[dn + 1]; ++e)
                    {
                      const int64_t c = elem_ids[e];
                      for (int q = 0; q < nq; ++q)
                        bm_add(bm, qb[c * nq + q]);
                    }
                }
            }
          __syncthreads();
          bm_extract(bm, nwords, IL, li, err);
        }
    }

    // nonIntList (bem_fma.cc:4669-4711): the parent's intList (sublevel 0) or
    // the box's previous sublevel's, childless entries not in the box's own
    // intList and the children not in it
    __global__ void __launch_bounds__(OT_THREADS)
      nil_kernel(int box0, int nbx, int L, int level, int nwords, BoxDev B,
                 const int32_t *__restrict__ lbase, ListStore IL, ListStore NIL, int *err)
    {
      extern __shared__ uint32_t bm[];
      uint32_t *own = bm + nwords; // the box's intList
      const int b   = box0 + blockIdx.x;
      if (blockIdx.x >= nbx)
        return;
      const int ns = B.nchild[b] == 0 ? L - level + 1 : 1;
      for (int sub = 0; sub < ns; ++sub)
        {
          bm_clear(bm, 2 * nwords);
          __syncthreads();
          const int li  = lbase[b] + sub;
          const int nil = IL.cnt[li];
          for (int e = threadIdx.x; e < nil; e += blockDim.x)
            bm_add(own, IL.ids[int64_t(li) * IL.cap + e]);
          __syncthreads();
          const int src = sub == 0 ? lbase[B.parent[b]] : li - 1;
          const int cn  = IL.cnt[src];
          for (int e = threadIdx.x; e < cn; e += blockDim.x)
            {
              const int pos = IL.ids[int64_t(src) * IL.cap + e];
              if (B.nchild[pos] == 0)
                {
                  if (!bm_has(own, pos))
                    bm_add(bm, pos);
                }
              else
                for (int c = 0; c < B.nchild[pos]; ++c)
                  if (!bm_has(own, B.child_first[pos] + c))
                    bm_add(bm, B.child_first[pos] + c);
            }
          __syncthreads();
          bm_extract(bm, nwords, NIL, li, err);
        }
    }
  } // namespace

  bool build_tree_device(const MeshHost &mesh, const double *d_xyz, const double *d_qpts, int nq,
                         int L, int max_nodes, const int32_t *d_dbl_off, const int32_t *d_dbl_ids,
                         const int32_t *d_elem_off, const int32_t *d_elem_ids, Tree &t,
                         cudaStream_t s)
  {
    const int64_t N = mesh.n_nodes;
    const int64_t Q = mesh.n_cells * nq;
    if (L < 1 || L > 20)
      throw Error(PIBEM_EINVAL, "Number of Octree Levels must be in 1..20");
    if (N + Q >= (int64_t(1) << 31))
      return false;
    t   = Tree();
    t.L = L;
    // root cube (bem_fma.cc:3713-3718)
    DBuf<unsigned long long> dmax;
    dmax.alloc(1);
    dmax.zero(s);
    absmax_kernel<<<std::min<unsigned>(nblk(3 * N), 1024), 256, 0, s>>>(3 * N, d_xyz, dmax.p);
    note_launch();
    unsigned long long bits = 0;
    dmax.download(&bits, 1, s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    double max_coor = 0;
    std::memcpy(&max_coor, &bits, sizeof(double));
    const double p0 = -1.1 * max_coor, delta0 = 2.2 * max_coor;

    // keys and sort
    DBuf<uint64_t> nk[2], qk[2];
    DBuf<int32_t>  nv[2], qv[2];
    for (int k = 0; k < 2; ++k)
      {
        nk[k].alloc(std::max<int64_t>(N, 1));
        nv[k].alloc(std::max<int64_t>(N, 1));
        qk[k].alloc(std::max<int64_t>(Q, 1));
        qv[k].alloc(std::max<int64_t>(Q, 1));
      }
    keys_kernel<<<nblk(N), 256, 0, s>>>(N, d_xyz, p0, delta0, L, nk[0].p, nv[0].p);
    if (Q > 0)
      keys_kernel<<<nblk(Q), 256, 0, s>>>(Q, d_qpts, p0, delta0, L, qk[0].p, qv[0].p);
    note_launch(2);
    DBuf<uint32_t> counts;
    auto sort = [&](int64_t n, DBuf<uint64_t> *k, DBuf<int32_t> *v) -> int {
      int cur = 0;
      if (n == 0)
        return 0;
      const int ntiles = int((n + RS_TILE - 1) / RS_TILE);
      counts.alloc(size_t(256) * ntiles);
      for (int shift = 0; shift < 3 * L; shift += 8)
        {
          rs_hist_kernel<<<ntiles, RS_THREADS, 0, s>>>(n, k[cur].p, shift, ntiles, counts.p);
          scan_kernel<<<1, 1024, 0, s>>>(int64_t(256) * ntiles, counts.p, nullptr);
          rs_scatter_kernel<<<ntiles, RS_THREADS, 0, s>>>(n, k[cur].p, v[cur].p, k[cur ^ 1].p,
                                                         v[cur ^ 1].p, shift, ntiles, counts.p);
          PIBEM_CUDA(cudaGetLastError());
          note_launch(3);
          cur ^= 1;
        }
      return cur;
    };
    const int nc = sort(N, nk, nv), qc = sort(Q, qk, qv);
    const uint64_t *nkey = nk[nc].p, *qkey = qk[qc].p;
    t.node_sorted.resize(N);
    t.quad_sorted.resize(Q);
    nv[nc].download(t.node_sorted.data(), N, s);
    if (Q > 0)
      qv[qc].download(t.quad_sorted.data(), Q, s);

    // levels
    auto add_box = [&](int lvl, int par, int dg, const double *pm, double d, const int *icp) {
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
      return int(t.level.size()) - 1;
    };
    {
      const double pm[3]  = {p0, p0, p0};
      const int    ic0[3] = {0, 0, 0};
      add_box(0, 0, 0, pm, delta0, ic0);
      t.nbeg = {0};
      t.nend = {int(N)};
      t.qbeg = {0};
      t.qend = {int(Q)};
    }
    t.startLevel.assign(L + 1, 0);
    t.endLevel.assign(L + 1, 0);
    t.dofs_filled.assign(L + 1, {});
    std::vector<double> weight(N);
    bool                unit_weights = true;
    for (int64_t i = 0; i < N; ++i)
      {
        const int ds = mesh.dbl_off[i + 1] - mesh.dbl_off[i];
        weight[i]    = 1.0 / double(ds);
        unit_weights = unit_weights && ds == 1;
      }
    DBuf<uint8_t>  nact, qact, dchildless;
    DBuf<int32_t>  ncur, qcur, dqbox, dbeg, dend;
    DBuf<uint32_t> flag, tot;
    DBuf<uint64_t> cmp, dpfx;
    nact.alloc(std::max<int64_t>(N, 1));
    qact.alloc(std::max<int64_t>(Q, 1));
    PIBEM_CUDA(cudaMemsetAsync(nact.p, 1, std::max<int64_t>(N, 1), s));
    PIBEM_CUDA(cudaMemsetAsync(qact.p, 1, std::max<int64_t>(Q, 1), s));
    ncur.alloc(std::max<int64_t>(N, 1));
    qcur.alloc(std::max<int64_t>(Q, 1));
    ncur.zero(s);
    qcur.zero(s);
    dqbox.alloc(std::max<int64_t>(size_t(L + 1) * Q, 1));
    PIBEM_CUDA(cudaMemsetAsync(dqbox.p, 0, sizeof(int32_t) * size_t(Q), s)); // level 0: the root
    flag.alloc(std::max<int64_t>(std::max(N, Q), 1));
    tot.alloc(1);
    cmp.alloc(std::max<int64_t>(std::max(N, Q), 1));
    // distinct prefixes of the active points of one array at a level
    auto prefixes = [&](int64_t n, const uint64_t *key, const uint8_t *act, int shift) {
      std::vector<uint64_t> out;
      if (n == 0)
        return out;
      run_start_kernel<<<nblk(n), 256, 0, s>>>(n, key, act, shift, flag.p);
      scan_kernel<<<1, 1024, 0, s>>>(n, flag.p, tot.p);
      run_compact_kernel<<<nblk(n), 256, 0, s>>>(n, key, act, shift, flag.p, cmp.p);
      PIBEM_CUDA(cudaGetLastError());
      note_launch(3);
      uint32_t cnt = 0;
      tot.download(&cnt, 1, s);
      PIBEM_CUDA(cudaStreamSynchronize(s));
      out.resize(cnt);
      if (cnt)
        cmp.download(out.data(), cnt, s);
      PIBEM_CUDA(cudaStreamSynchronize(s));
      return out;
    };
    std::vector<int>      parents = {0};
    std::vector<uint64_t> parent_pfx = {0};
    double                d = delta0;
    for (int l = 1; l <= L; ++l)
      {
        d /= 2.;
        const int             shift = 3 * (L - l);
        std::vector<uint64_t> pn = prefixes(N, nkey, nact.p, shift), pq = prefixes(Q, qkey, qact.p, shift);
        std::vector<uint64_t> pf;
        pf.reserve(pn.size() + pq.size());
        std::merge(pn.begin(), pn.end(), pq.begin(), pq.end(), std::back_inserter(pf));
        pf.erase(std::unique(pf.begin(), pf.end()), pf.end());
        const int nbx  = int(pf.size());
        const int box0 = int(t.level.size());
        t.startLevel[l] = box0;
        t.endLevel[l]   = box0 + nbx - 1;
        std::vector<int32_t> nb(nbx), ne(nbx), qb(nbx), qe(nbx);
        if (nbx > 0)
          {
            dpfx.upload(pf, s);
            dbeg.alloc(size_t(4) * nbx);
            dend.alloc(size_t(4) * nbx);
            box_range_kernel<<<nblk(nbx), 256, 0, s>>>(nbx, dpfx.p, shift, N, nkey, dbeg.p, dend.p);
            box_range_kernel<<<nblk(nbx), 256, 0, s>>>(nbx, dpfx.p, shift, Q, qkey, dbeg.p + nbx,
                                                       dend.p + nbx);
            note_launch(2);
            std::vector<int32_t> bb(2 * size_t(nbx)), be(2 * size_t(nbx));
            dbeg.download(bb.data(), bb.size(), s);
            dend.download(be.data(), be.size(), s);
            PIBEM_CUDA(cudaStreamSynchronize(s));
            std::copy(bb.begin(), bb.begin() + nbx, nb.begin());
            std::copy(bb.begin() + nbx, bb.end(), qb.begin());
            std::copy(be.begin(), be.begin() + nbx, ne.begin());
            std::copy(be.begin() + nbx, be.end(), qe.begin());
          }
        // box records: parent by the prefix without its last digit
        std::vector<uint8_t> cl(std::max(nbx, 1), 0);
        std::vector<int>     next;
        size_t               pi = 0;
        for (int k = 0; k < nbx; ++k)
          {
            const uint64_t pp = pf[k] >> 3;
            while (pi < parent_pfx.size() && parent_pfx[pi] < pp)
              ++pi;
            if (pi >= parent_pfx.size() || parent_pfx[pi] != pp)
              throw Error(PIBEM_ECUDA, "internal error: octree box without its parent");
            const int P  = parents[pi];
            const int dg = int(pf[k] & 7u);
            double    pm[3];
            int       icc[3];
            static const int coff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                           {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
            for (int c = 0; c < 3; ++c)
              {
                pm[c]  = coff[dg][c] ? t.pmin[3 * P + c] + d : t.pmin[3 * P + c];
                icc[c] = 2 * t.ic[3 * P + c] + coff[dg][c];
              }
            const int id = add_box(l, P, dg, pm, d, icc);
            t.nbeg.push_back(nb[k]);
            t.nend.push_back(ne[k]);
            t.qbeg.push_back(qb[k]);
            t.qend.push_back(qe[k]);
            if (t.nchild[P] == 0)
              t.child_first[P] = id;
            t.nchild[P]++;
            // childless test: node weights summed in ascending node order
            double numNodes = 0.0;
            if (unit_weights)
              numNodes = double(ne[k] - nb[k]);
            else
              {
                std::vector<int> ids(t.node_sorted.begin() + nb[k], t.node_sorted.begin() + ne[k]);
                std::sort(ids.begin(), ids.end());
                for (int i : ids)
                  numNodes += weight[i];
              }
            // a box that fails the test at the deepest level is childless too
            // and joins the list after the loop, as in the reference
            const bool pass = std::round(numNodes) <= max_nodes;
            if (pass)
              t.childless.push_back(id);
            else
              next.push_back(id);
            cl[k] = pass || l == L;
            if (numNodes > 0)
              t.dofs_filled[l].push_back(id);
          }
        if (nbx > 0)
          {
            dchildless.upload(cl, s);
            assign_kernel<<<nblk(N), 256, 0, s>>>(N, nkey, nact.p, shift, nbx, dpfx.p, box0,
                                                  dchildless.p, ncur.p);
            if (Q > 0)
              {
                assign_kernel<<<nblk(Q), 256, 0, s>>>(Q, qkey, qact.p, shift, nbx, dpfx.p, box0,
                                                      dchildless.p, qcur.p);
                qbox_kernel<<<nblk(Q), 256, 0, s>>>(Q, qv[qc].p, qcur.p, dqbox.p + size_t(l) * Q);
              }
            note_launch(3);
          }
        else if (Q > 0)
          {
            qbox_kernel<<<nblk(Q), 256, 0, s>>>(Q, qv[qc].p, qcur.p, dqbox.p + size_t(l) * Q);
            note_launch();
          }
        parents.swap(next);
        parent_pfx.clear();
        for (int b : parents)
          {
            const int k = b - box0;
            parent_pfx.push_back(pf[k]);
          }
      }
    for (int b : parents)
      t.childless.push_back(b);
    t.nb = int(t.level.size());
    t.is_childless.assign(t.nb, 0);
    for (int b : t.childless)
      t.is_childless[b] = 1;
    t.qbox.resize(size_t(L + 1) * Q);
    if (Q > 0)
      dqbox.download(t.qbox.data(), t.qbox.size(), s);
    t.node_leaf.assign(N, -1);
    {
      std::vector<int32_t> nl(N);
      ncur.download(nl.data(), N, s);
      PIBEM_CUDA(cudaStreamSynchronize(s));
      for (int64_t k = 0; k < N; ++k)
        t.node_leaf[t.node_sorted[k]] = nl[k];
    }

    // ---- lists
    const int nbt = t.nb;
    std::vector<int32_t> lbase(nbt + 1, 0);
    for (int b = 0; b < nbt; ++b)
      lbase[b + 1] = lbase[b] + ((t.nchild[b] == 0 && t.level[b] >= 2) ? L - t.level[b] + 1 : 1);
    const int nlists = lbase[nbt];
    const int CAP_NN = 512, CAP_IL = 1024, CAP_NIL = 2048;
    DBuf<int32_t> d_lbase, d_nn, d_il, d_nil, c_nn, c_il, c_nil, d_nchild, d_cfirst, d_parent,
      d_nbeg, d_nend;
    DBuf<double> d_pmin, d_delta;
    DBuf<int>    d_err;
    d_lbase.upload(lbase, s);
    d_nn.alloc(size_t(nlists) * CAP_NN);
    d_il.alloc(size_t(nlists) * CAP_IL);
    d_nil.alloc(size_t(nlists) * CAP_NIL);
    c_nn.alloc(nlists);
    c_il.alloc(nlists);
    c_nil.alloc(nlists);
    c_nn.zero(s);
    c_il.zero(s);
    c_nil.zero(s);
    d_nchild.upload(t.nchild, s);
    d_cfirst.upload(t.child_first, s);
    d_parent.upload(t.parent, s);
    d_nbeg.upload(t.nbeg, s);
    d_nend.upload(t.nend, s);
    d_pmin.upload(t.pmin, s);
    d_delta.upload(t.delta, s);
    d_err.alloc(1);
    d_err.zero(s);
    // level 1: nearNeigh = intList = the level-1 boxes; nonIntList empty
    {
      std::vector<int32_t> lvl1;
      for (int b = t.startLevel[1]; b <= t.endLevel[1]; ++b)
        lvl1.push_back(b);
      std::vector<int32_t> ids(size_t(lvl1.size()) * CAP_NN), cnt(lvl1.size(), int(lvl1.size()));
      if (lvl1.size() > size_t(CAP_NN))
        return false;
      for (size_t k = 0; k < lvl1.size(); ++k)
        {
          std::copy(lvl1.begin(), lvl1.end(), ids.begin() + k * CAP_NN);
          PIBEM_CUDA(cudaMemcpyAsync(d_nn.p + size_t(lbase[lvl1[k]]) * CAP_NN, ids.data() + k * CAP_NN,
                                     sizeof(int32_t) * lvl1.size(), cudaMemcpyHostToDevice, s));
          PIBEM_CUDA(cudaMemcpyAsync(d_il.p + size_t(lbase[lvl1[k]]) * CAP_IL, ids.data() + k * CAP_NN,
                                     sizeof(int32_t) * lvl1.size(), cudaMemcpyHostToDevice, s));
          PIBEM_CUDA(cudaMemcpyAsync(c_nn.p + lbase[lvl1[k]], cnt.data(), sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
          PIBEM_CUDA(cudaMemcpyAsync(c_il.p + lbase[lvl1[k]], cnt.data(), sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        }
      PIBEM_CUDA(cudaStreamSynchronize(s)); // the host staging above goes out of scope
    }
    // box-id bitmaps of the list kernels in shared memory (two for nonIntList)
    const int    nwords   = (nbt + 31) / 32;
    const size_t bm_bytes = size_t(nwords) * sizeof(uint32_t);
    if (2 * bm_bytes > 200 * 1024)
      return false;
    if (2 * bm_bytes > 48 * 1024)
      {
        raise_smem_limit(reinterpret_cast<const void *>(nil_kernel), 2 * bm_bytes);
        raise_smem_limit(reinterpret_cast<const void *>(il_kernel), bm_bytes);
        raise_smem_limit(reinterpret_cast<const void *>(nn_kernel), bm_bytes);
      }
    BoxDev B{d_pmin.p, d_delta.p, d_nchild.p, d_cfirst.p, d_parent.p, d_nbeg.p, d_nend.p};
    ListStore NN{d_nn.p, c_nn.p, CAP_NN}, IL{d_il.p, c_il.p, CAP_IL}, NIL{d_nil.p, c_nil.p, CAP_NIL};
    for (int l = 2; l <= L; ++l)
      {
        const int b0 = t.startLevel[l], nbx = t.endLevel[l] - b0 + 1;
        if (nbx <= 0)
          continue;
        nn_kernel<<<nbx, OT_THREADS, bm_bytes, s>>>(b0, nbx, L, l, nwords, B, d_lbase.p, NN, d_err.p);
        il_kernel<<<nbx, OT_THREADS, bm_bytes, s>>>(b0, nbx, L, l, nwords, B, d_lbase.p, nv[nc].p,
                                                    d_dbl_off, d_dbl_ids, d_elem_off, d_elem_ids, nq,
                                                    Q, dqbox.p, NN, IL, d_err.p);
        nil_kernel<<<nbx, OT_THREADS, 2 * bm_bytes, s>>>(b0, nbx, L, l, nwords, B, d_lbase.p, IL, NIL,
                                                         d_err.p);
        PIBEM_CUDA(cudaGetLastError());
        note_launch(3);
      }
    int err = 0;
    d_err.download(&err, 1, s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    if (err)
      return false;
    // download the lists into the nested form the plan reads
    std::vector<int32_t> cn(nlists), ci(nlists), cx(nlists);
    c_nn.download(cn.data(), nlists, s);
    c_il.download(ci.data(), nlists, s);
    c_nil.download(cx.data(), nlists, s);
    std::vector<int32_t> hn(size_t(nlists) * CAP_NN), hi(size_t(nlists) * CAP_IL),
      hx(size_t(nlists) * CAP_NIL);
    d_nn.download(hn.data(), hn.size(), s);
    d_il.download(hi.data(), hi.size(), s);
    d_nil.download(hx.data(), hx.size(), s);
    PIBEM_CUDA(cudaStreamSynchronize(s));
    t.nn.assign(nbt, {});
    t.il.assign(nbt, {});
    t.nil.assign(nbt, {});
    for (int b = 0; b < nbt; ++b)
      {
        const int ns = lbase[b + 1] - lbase[b];
        t.nn[b].resize(ns);
        t.il[b].resize(ns);
        t.nil[b].resize(ns);
        if (t.level[b] == 0)
          continue;
        for (int sub = 0; sub < ns; ++sub)
          {
            const int li = lbase[b] + sub;
            t.nn[b][sub].assign(hn.begin() + size_t(li) * CAP_NN, hn.begin() + size_t(li) * CAP_NN + cn[li]);
            t.il[b][sub].assign(hi.begin() + size_t(li) * CAP_IL, hi.begin() + size_t(li) * CAP_IL + ci[li]);
            t.nil[b][sub].assign(hx.begin() + size_t(li) * CAP_NIL,
                                 hx.begin() + size_t(li) * CAP_NIL + cx[li]);
          }
      }
    return true;
  }
} // namespace pibem

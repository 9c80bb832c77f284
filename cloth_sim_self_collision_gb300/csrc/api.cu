// api.cu -- the C ABI (include/clothgpu.h): contexts, the device arena of
// cloths, and the host orchestration of the frame
// (self_contact_sparse/main.cpp:213-263).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <tuple>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ctx.h"

using namespace cs;

namespace cs {
namespace host {

int slot_of(cs_ctx* c, int id) {
  for (size_t i = 0; i < c->order.size(); i++)
    if (c->order[i] == id) return (int)i;
  throw ArgError("unknown cloth id " + std::to_string(id));
}

DevParams to_dev(const cs_params& p) {
  DevParams d;
  static_assert(sizeof(DevParams) == sizeof(cs_params), "parameter layouts differ");
  std::memcpy(&d, &p, sizeof(d));
  return d;
}

void free_contacts(cs_ctx* c) {
  c->cmem.release();
  c->C = ContactBufs();
}

// q_fv / q_ee: queue capacities of the narrow phase (-1: derived from pair_cap)
void alloc_contacts_into(const Arena& A, ContactBufs& C, DevMem& m, cudaStream_t s, int pair_cap, int cand_cap,
                         int q_fv = -1, int q_ee = -1) {
  C.pair_cap = pair_cap;
  C.cand_cap = cand_cap;
  C.ce_cap = cand_cap;
  C.pairs = m.alloc<int2>(pair_cap);
  C.q_cap[0] = q_fv > 0 ? q_fv : std::max(pair_cap / 2, 4096);
  C.q_cap[1] = q_ee > 0 ? q_ee : (int)std::min<long long>(2LL * pair_cap, 0x7fffffffLL);
  C.queue[0] = m.alloc<int2>(C.q_cap[0]);
  C.queue[1] = m.alloc<int2>(C.q_cap[1]);
  C.queue64[0] = m.alloc<int2>(C.q_cap[0]);
  C.queue64[1] = m.alloc<int2>(C.q_cap[1]);
  C.cand = m.alloc<Cand>(cand_cap);
  C.cand_sorted = m.alloc<Cand>(cand_cap);
  C.key_a = m.alloc<unsigned long long>(cand_cap);
  C.key_b = m.alloc<unsigned long long>(cand_cap);
  C.idx_a = m.alloc<int>(cand_cap);
  C.idx_b = m.alloc<int>(cand_cap);
  C.ce = m.alloc<int>(5 * (size_t)cand_cap);
  C.ce_inst_lo = m.alloc<int>(A.ni);
  C.ce_inst_hi = m.alloc<int>(A.ni);
  C.counters = m.alloc<int>(16);
  C.level = m.alloc<int>(cand_cap);
  C.order = m.alloc<int>(cand_cap);
  C.imp_pre = m.alloc<double>(9 * (size_t)cand_cap);
  C.lev_cnt = m.alloc<int>((size_t)cand_cap + A.ni + 1);
  C.vmark = m.alloc<int>(A.nv);
  C.vstamp = m.alloc<int>(A.nv);
  C.zkey = m.alloc<unsigned long long>(A.nv);
  C.zkey2 = m.alloc<unsigned long long>(A.nv);
  C.zrec = m.alloc<double>(9 * (size_t)A.nv);
  C.cub_bytes = cub_sort_bytes(std::max(cand_cap, A.nv));
  C.cub_tmp = m.alloc<char>(C.cub_bytes);
  CK(cudaMemsetAsync(C.vstamp, 0xff, sizeof(int) * (size_t)A.nv, s));
  CK(cudaMemsetAsync(C.counters, 0, sizeof(int) * 16, s));
}

void alloc_contacts(cs_ctx* c, int pair_cap, int cand_cap, int q_fv = -1, int q_ee = -1) {
  graph_release(c);  // the graph holds the old buffers' addresses
  free_contacts(c);
  alloc_contacts_into(c->A, c->C, c->cmem, c->stream, pair_cap, cand_cap, q_fv, q_ee);
}

// Packs the cloths cl (in this order) into a fresh device arena o on stream s:
// global indices, slot lists, BVH, SELL slices, and the cloths' host states.
// Reads only the cloths, so it may run on another thread while a context
// steps its current arena.
void build_arena(ArenaSet& o, const std::vector<const Cloth*>& cl, cudaStream_t s) {
  Arena A;
  const int ni = (int)cl.size();
  o.order.clear();
  for (const Cloth* k : cl) o.order.push_back(k->id);
  A.ni = ni;
  o.voff.assign(ni + 1, 0);
  o.toff.assign(ni + 1, 0);
  o.qoff.assign(ni + 1, 0);
  o.boff.assign(ni + 1, 0);
  o.noff.assign(ni + 1, 0);
  o.solver.assign(ni, 0);
  std::vector<int> eoff(ni + 1, 0), chunk_off(ni + 1, 0);
  for (int i = 0; i < ni; i++) {
    const ClothTopo& t = cl[i]->topo;
    o.voff[i + 1] = o.voff[i] + t.np;
    o.toff[i + 1] = o.toff[i] + t.nt;
    o.qoff[i + 1] = o.qoff[i] + t.nq;
    o.boff[i + 1] = o.boff[i] + t.nb;
    o.noff[i + 1] = o.noff[i] + t.nnode;
    eoff[i + 1] = eoff[i] + (int)t.edge_uv.size() / 2;
    chunk_off[i + 1] = chunk_off[i] + (t.np + 255) / 256;
    o.solver[i] = cl[i]->prm.solver_kind;
  }
  A.nv = o.voff[ni];
  A.nt = o.toff[ni];
  A.nq = o.qoff[ni];
  A.nb = o.boff[ni];
  A.nn = o.noff[ni];
  A.ne = eoff[ni];
  A.nchunk = chunk_off[ni];
  const int NV = A.nv, NT = A.nt, NQ = A.nq, NB = A.nb, NN = A.nn;
  std::vector<double> X0, x, v;
  std::vector<int> bc, vinst, tri, tinst, quad, qinst, row_ptr, col_idx, dia_split, blk_row;
  std::vector<int> slot_ptr(1, 0), slot_src, grad_ptr(1, 0), grad_src;
  std::vector<int> lev_off(1, 0), lev_ptr(1, 0), lev_rows, blev_off(1, 0), blev_ptr(1, 0), blev_rows;
  std::vector<int> fac_ptr(1, 0), fac_ops;
  std::vector<int> node, pre, skip, leaf_lo, leaf_hi, depth, prepos(NN), tri_leaf(NT), edge_uv;
  std::vector<int> chunk_inst, chunk_lo(ni), chunk_hi(ni);
  std::vector<DevParams> prm;
  X0.reserve(3 * (size_t)NV);
  for (int i = 0; i < ni; i++) {
    const Cloth& ci = *cl[i];
    const ClothTopo& t = ci.topo;
    const int vo = o.voff[i], to = o.toff[i], qo = o.qoff[i], bo = o.boff[i], no = o.noff[i];
    prm.push_back(to_dev(ci.prm));
    X0.insert(X0.end(), t.X0.begin(), t.X0.end());
    x.insert(x.end(), ci.x.begin(), ci.x.end());
    v.insert(v.end(), ci.v.begin(), ci.v.end());
    bc.insert(bc.end(), t.bc.begin(), t.bc.end());
    vinst.insert(vinst.end(), t.np, i);
    for (int k : t.tri) tri.push_back(k + vo);
    tinst.insert(tinst.end(), t.nt, i);
    for (int k : t.quad) quad.push_back(k + vo);
    qinst.insert(qinst.end(), t.nq, i);
    for (int r = 0; r < t.np; r++) {
      row_ptr.push_back(t.row_ptr[r] + bo);
      dia_split.push_back(t.dia_split[r] + bo);
      for (int s = t.row_ptr[r]; s < t.row_ptr[r + 1]; s++) blk_row.push_back(r + vo);
    }
    for (int k : t.col_idx) col_idx.push_back(k + vo);
    for (int k = 0; k < (int)t.edge_uv.size(); k++) edge_uv.push_back(t.edge_uv[k] + vo);
    for (int k = chunk_off[i]; k < chunk_off[i + 1]; k++) chunk_inst.push_back(i);
    chunk_lo[i] = chunk_off[i];
    chunk_hi[i] = chunk_off[i + 1];
    // BVH
    for (int n = 0; n < t.nnode; n++) {
      const int par = t.node[3 * n], c0 = t.node[3 * n + 1], c1 = t.node[3 * n + 2];
      node.push_back(par < 0 ? -1 : par + no);
      if (c1 == -1) {
        node.push_back(c0 + to);
        node.push_back(-1);
        tri_leaf[c0 + to] = n + no;
      } else {
        node.push_back(c0 + no);
        node.push_back(c1 + no);
      }
      leaf_lo.push_back(t.leaf_lo[n]);
      leaf_hi.push_back(t.leaf_hi[n]);
      depth.push_back(t.depth[n]);
    }
    for (int k = 0; k < t.nnode; k++) {
      pre.push_back(t.pre[k] + no);
      skip.push_back(t.skip[k] + no);
      prepos[t.pre[k] + no] = k;
    }
    // ILU level tables (rows global)
    if (!t.lev_ptr.empty()) {
      const int rb = lev_ptr.back();
      for (size_t l = 1; l < t.lev_ptr.size(); l++) lev_ptr.push_back(rb + t.lev_ptr[l]);
      for (int r : t.lev_rows) lev_rows.push_back(r + vo);
      const int rbb = blev_ptr.back();
      for (size_t l = 1; l < t.blev_ptr.size(); l++) blev_ptr.push_back(rbb + t.blev_ptr[l]);
      for (int r : t.blev_rows) blev_rows.push_back(r + vo);
    }
    lev_off.push_back((int)lev_ptr.size() - 1);
    blev_off.push_back((int)blev_ptr.size() - 1);
    const int fb = fac_ptr.back();
    for (int r = 0; r < t.np; r++) fac_ptr.push_back(fb + (t.fac_ptr.empty() ? 0 : t.fac_ptr[r + 1]));
    for (size_t k = 0; k < t.fac_ops.size(); k += 3) {
      fac_ops.push_back(t.fac_ops[k] + bo);
      fac_ops.push_back(t.fac_ops[k + 1] + bo);
      fac_ops.push_back(t.fac_ops[k + 2] < 0 ? -1 : t.fac_ops[k + 2] + bo);
    }
  }
  row_ptr.push_back(NB);
  // slot lists: every cloth's off-diagonal slots, then every cloth's diagonal slots
  auto glob = [&](int i, int code, int per_tri, int per_quad) {
    return code >= 0 ? code + o.toff[i] * per_tri : -((-code - 1) + o.qoff[i] * per_quad) - 1;
  };
  for (int i = 0; i < ni; i++) {
    const ClothTopo& t = cl[i]->topo;
    for (int s = 0; s < t.nb; s++) {
      for (int e = t.slot_ptr[s]; e < t.slot_ptr[s + 1]; e++) slot_src.push_back(glob(i, t.slot_src[e], 9, 16));
      slot_ptr.push_back((int)slot_src.size());
    }
  }
  for (int i = 0; i < ni; i++) {
    const ClothTopo& t = cl[i]->topo;
    for (int s = t.nb; s < t.nb + t.np; s++) {
      for (int e = t.slot_ptr[s]; e < t.slot_ptr[s + 1]; e++) slot_src.push_back(glob(i, t.slot_src[e], 9, 16));
      slot_ptr.push_back((int)slot_src.size());
    }
    for (int r = 0; r < t.np; r++) {
      for (int e = t.grad_ptr[r]; e < t.grad_ptr[r + 1]; e++) grad_src.push_back(glob(i, t.grad_src[e], 3, 4));
      grad_ptr.push_back((int)grad_src.size());
    }
  }
  DevMem& m = o.mem;
  std::vector<int> ones(ni, 1);
  A.active = m.upload(ones, s);
  A.voff = m.upload(o.voff, s);
  A.toff = m.upload(o.toff, s);
  A.qoff = m.upload(o.qoff, s);
  A.boff = m.upload(o.boff, s);
  A.noff = m.upload(o.noff, s);
  A.preoff = A.noff;
  A.chunk_lo = m.upload(chunk_lo, s);
  A.chunk_hi = m.upload(chunk_hi, s);
  A.chunk_inst = m.upload(chunk_inst, s);
  A.prm = m.upload(prm, s);
  A.st = m.alloc<InstState>(ni);
  CK(cudaMemsetAsync(A.st, 0, sizeof(InstState) * (size_t)std::max(ni, 1), s));
  A.X0 = m.upload(X0, s);
  A.x = m.upload(x, s);
  A.v = m.upload(v, s);
  A.x1 = m.alloc<double>(3 * (size_t)NV);
  A.v0 = m.alloc<double>(3 * (size_t)NV);
  A.bc = m.upload(bc, s);
  A.vinst = m.upload(vinst, s);
  A.tri = m.upload(tri, s);
  A.tinst = m.upload(tinst, s);
  A.quad = m.upload(quad, s);
  A.qinst = m.upload(qinst, s);
  A.qK = m.alloc<double>(4 * (size_t)NQ);
  A.qscale = m.alloc<double>(NQ);
  A.tri_blk = m.alloc<double>(81 * (size_t)NT);
  A.tri_grad = m.alloc<double>(9 * (size_t)NT);
  A.quad_grad = m.alloc<double>(12 * (size_t)NQ);
  A.row_ptr = m.upload(row_ptr, s);
  A.col_idx = m.upload(col_idx, s);
  A.dia_split = m.upload(dia_split, s);
  A.blk_row = m.upload(blk_row, s);
  A.slot_ptr = m.upload(slot_ptr, s);
  A.slot_src = m.upload(slot_src, s);
  A.grad_ptr = m.upload(grad_ptr, s);
  A.grad_src = m.upload(grad_src, s);
  A.vdia = m.alloc<double>(9 * (size_t)NV);
  A.vcrs = m.alloc<double>(9 * (size_t)NB);
  A.fdia = m.alloc<double>(9 * (size_t)NV);
  A.fcrs = m.alloc<double>(9 * (size_t)NB);
  A.b = m.alloc<double>(3 * (size_t)NV);
  A.r = m.alloc<double>(3 * (size_t)NV);
  A.p = m.alloc<double>(3 * (size_t)NV);
  A.z = m.alloc<double>(3 * (size_t)NV);
  A.dx = m.alloc<double>(3 * (size_t)NV);
  if (NV > 0) CK(cudaMemsetAsync(A.z, 0, sizeof(double) * 3 * (size_t)NV, s));
  A.part = m.alloc<double>(2 * (size_t)A.nchunk);
  {
    std::vector<long long> cb(A.nchunk, 0);
    for (int k = 0; k < A.nchunk; k++) {
      const int i = chunk_inst[k];
      const ClothTopo& t = cl[i]->topo;
      const int r0 = (k - chunk_lo[i]) * 256;
      for (int l = 0; l < 256 && r0 + l < t.np; l++)
        cb[k] += 76LL * (t.row_ptr[r0 + l + 1] - t.row_ptr[r0 + l]) + 72 + 48 + 4;  // blocks + cols, diag, x, y, row ptr
    }
    A.chunk_bytes = m.upload(cb, s);
    A.bytes_acc = m.alloc<unsigned long long>(8);
    CK(cudaMemsetAsync(A.bytes_acc, 0, 8 * sizeof(unsigned long long), s));
  }
  A.lev_off = m.upload(lev_off, s);
  A.lev_ptr = m.upload(lev_ptr, s);
  A.lev_rows = m.upload(lev_rows, s);
  A.blev_off = m.upload(blev_off, s);
  A.blev_ptr = m.upload(blev_ptr, s);
  A.blev_rows = m.upload(blev_rows, s);
  A.fac_ptr = m.upload(fac_ptr, s);
  A.fac_ops = m.upload(fac_ops, s);
  A.sing = m.alloc<int>(NV);
  A.node = m.upload(node, s);
  A.pre = m.upload(pre, s);
  A.skip = m.upload(skip, s);
  A.leaf_lo = m.upload(leaf_lo, s);
  A.leaf_hi = m.upload(leaf_hi, s);
  A.depth = m.upload(depth, s);
  A.prepos = m.upload(prepos, s);
  A.tri_leaf = m.upload(tri_leaf, s);
  A.refit_cnt = m.alloc<int>(NN);
  A.box = m.alloc<Box>(NN);
  A.box32 = m.alloc<float>(6 * (size_t)NN);
  A.vb32 = m.alloc<float>(6 * (size_t)NV);
  A.edge_uv = m.upload(edge_uv, s);
  A.vdirty = m.alloc<int>(NV);
  A.ccd32 = m.alloc<float4>(3 * (size_t)NV);
  A.tdirty = m.alloc<int>(NT);
  CK(cudaMemsetAsync(A.tdirty, 0, sizeof(int) * (size_t)std::max(NT, 1), s));
  A.uf = m.alloc<int>(NV);
  A.inzone = m.alloc<int>(NV);
  CK(cudaMemsetAsync(A.inzone, 0, sizeof(int) * (size_t)std::max(NV, 1), s));
  o.d_list = m.alloc<int>(std::max(ni, 1));
  A.ctl = m.alloc<FrameCtl>(1);
  CK(cudaMemsetAsync(A.ctl, 0, sizeof(FrameCtl), s));
  // mixed precision: SELL-32 slices of every cloth's rows (32 rows per slice,
  // padded to the widest row with zero blocks pointing at the slice's own row)
  {
    std::vector<int> slice_inst, slice_row0, slice_w, slice_lo(ni), slice_hi(ni), col32;
    std::vector<long long> slice_voff, slice_coff, sell_pos((size_t)NB + NV);
    long long vtot = 0, ctot = 0;
    for (int i = 0; i < ni; i++) {
      const ClothTopo& t = cl[i]->topo;
      const int vo = o.voff[i], bo = o.boff[i];
      slice_lo[i] = (int)slice_inst.size();
      for (int r0 = 0; r0 < t.np; r0 += 32) {
        const int n = std::min(32, t.np - r0);
        int w = 0;
        for (int l = 0; l < n; l++) w = std::max(w, t.row_ptr[r0 + l + 1] - t.row_ptr[r0 + l] + 1);
        slice_inst.push_back(i);
        slice_row0.push_back(vo + r0);
        slice_w.push_back(w);
        slice_voff.push_back(vtot);
        slice_coff.push_back(ctot);
        for (int j = 0; j < w; j++)
          for (int l = 0; l < 32; l++) {
            int col = vo + r0;
            if (l < n) {
              const int row = r0 + l, len = t.row_ptr[row + 1] - t.row_ptr[row];
              col = (j < len) ? t.col_idx[t.row_ptr[row] + j] + vo : vo + row;
              if (j < len) sell_pos[(size_t)bo + t.row_ptr[row] + j] = vtot + 9LL * 32 * j + l;
              if (j == len) sell_pos[(size_t)NB + vo + row] = vtot + 9LL * 32 * j + l;
            }
            col32.push_back(col);
          }
        vtot += 9LL * 32 * w;
        ctot += 32LL * w;
      }
      slice_hi[i] = (int)slice_inst.size();
    }
    A.nslice = (int)slice_inst.size();
    A.slice_inst = m.upload(slice_inst, s);
    A.slice_row0 = m.upload(slice_row0, s);
    A.slice_w = m.upload(slice_w, s);
    A.slice_lo = m.upload(slice_lo, s);
    A.slice_hi = m.upload(slice_hi, s);
    A.slice_voff = m.upload(slice_voff, s);
    A.slice_coff = m.upload(slice_coff, s);
    A.sell_pos = m.upload(sell_pos, s);
    A.col32 = m.upload(col32, s);
    A.val32 = m.alloc<float>(vtot);
    CK(cudaMemsetAsync(A.val32, 0, sizeof(float) * (size_t)std::max(vtot, 1LL), s));
    A.linv32 = m.alloc<float>(9 * (size_t)NV);
    A.r32 = m.alloc<float>(4 * (size_t)NV);
    A.r32b = m.alloc<float>(4 * (size_t)NV);
    A.w32 = m.alloc<float>(4 * (size_t)NV);
    A.w32b = m.alloc<float>(4 * (size_t)NV);
    A.s32 = m.alloc<float>(4 * (size_t)NV);
    A.s32b = m.alloc<float>(4 * (size_t)NV);
    A.d32 = m.alloc<float>(4 * (size_t)NV);
    A.p32 = m.alloc<float>(4 * (size_t)NV);
    A.q32 = m.alloc<float>(4 * (size_t)NV);
    A.z32 = m.alloc<float>(4 * (size_t)NV);
    A.part32 = m.alloc<double>(3 * (size_t)std::max(A.nslice, 1));
    {
      std::vector<long long> sb(A.nslice, 0);
      for (int k = 0; k < A.nslice; k++) {
        const int i = slice_inst[k];
        const ClothTopo& t = cl[i]->topo;
        const int r0 = slice_row0[k] - o.voff[i];
        for (int l = 0; l < 32 && r0 + l < t.np; l++)
          sb[k] += 40LL * (t.row_ptr[r0 + l + 1] - t.row_ptr[r0 + l] + 1) + 24;  // blocks + cols, x, y (FP32)
      }
      A.slice_bytes = m.upload(sb, s);
    }
    A.red_cnt = m.alloc<int>(std::max(ni, 1));
    CK(cudaMemsetAsync(A.red_cnt, 0, sizeof(int) * (size_t)std::max(ni, 1), s));
    // persistent inner solve: algorithmic bytes of one iteration over a slice
    // (blocks and columns; r, w, s_prev, p_prev and d read; s, r_next, w_next, p
    // and d written)
    {
      std::vector<long long> pb(A.nslice, 0);
      for (int k = 0; k < A.nslice; k++) {
        const int i = slice_inst[k];
        const ClothTopo& t = cl[i]->topo;
        const int r0 = slice_row0[k] - o.voff[i];
        for (int l = 0; l < 32 && r0 + l < t.np; l++)
          pb[k] += 40LL * (t.row_ptr[r0 + l + 1] - t.row_ptr[r0 + l] + 1) + 120;
      }
      A.slice_pbytes = m.upload(pb, s);
      A.dg_range = m.alloc<unsigned>(2 * (size_t)std::max(ni, 1));
      A.grid_bar = m.alloc<unsigned int>(8);
      CK(cudaMemsetAsync(A.grid_bar, 0, 8 * sizeof(unsigned int), s));
    }
    A.mixed = 1;
  }
  o.A = A;
  if (ni > 0) launch_quad_factors(A, s);
  alloc_contacts_into(o.A, o.C, o.cmem, s, 16 * NT + 4096, 4 * NT + 4096);
  CK(cudaStreamSynchronize(s));
  CK(cudaGetLastError());
  o.hst.assign(ni, InstState());
}

// Makes o the context's arena; the previous arena's buffers end up in o.
void install(cs_ctx* c, ArenaSet& o) {
  graph_release(c);
  o.A.narrow_regs = c->narrow_regs;
  o.A.bar_sleep_ns = c->bar_sleep_ns;
  o.A.impulse_cluster = c->impulse_cluster;
  o.A.mx_eta_big = c->mx_eta_big;
  o.A.bar_timeout_ns = c->bar_timeout_ns;
  o.A.bar_hold = c->bar_hold;
  std::swap(c->A, o.A);
  std::swap(c->C, o.C);
  std::swap(c->mem, o.mem);
  std::swap(c->cmem, o.cmem);
  std::swap(c->order, o.order);
  std::swap(c->voff, o.voff);
  std::swap(c->toff, o.toff);
  std::swap(c->qoff, o.qoff);
  std::swap(c->boff, o.boff);
  std::swap(c->noff, o.noff);
  std::swap(c->solver, o.solver);
  std::swap(c->d_list, o.d_list);
  std::swap(c->hst, o.hst);
  c->dead.assign(c->order.size(), 0);
  for (size_t i = 0; i < c->order.size(); i++) c->dead[i] = c->cloths[c->order[i]]->stats.diverged;
  c->last_ncand = 0;
  c->last_nce = 0;
  c->dirty = false;
}

// Rebuilds the device arena from c->order, keeping the cloths' (saved) states.
void rebuild(cs_ctx* c) {
  if (!c->dirty) return;
  c->mem.release();
  free_contacts(c);
  std::vector<const Cloth*> cl;
  for (int id : c->order) cl.push_back(c->cloths[id].get());
  ArenaSet o;
  build_arena(o, cl, c->stream);
  install(c, o);
}

// copies resident states back to the cloths before the arena changes
void save_states(cs_ctx* c) {
  if (c->dirty || c->order.empty()) return;
  for (size_t i = 0; i < c->order.size(); i++) {
    Cloth& cl = *c->cloths[c->order[i]];
    CK(cudaMemcpyAsync(cl.x.data(), c->A.x + 3 * (size_t)c->voff[i], sizeof(double) * cl.x.size(),
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(cl.v.data(), c->A.v + 3 * (size_t)c->voff[i], sizeof(double) * cl.v.size(),
                       cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
}

// act without the cloths that blew up
std::vector<int> live(const cs_ctx* c, const std::vector<int>& act) {
  std::vector<int> a = act;
  for (size_t i = 0; i < a.size() && i < c->dead.size(); i++)
    if (c->dead[i]) a[i] = 0;
  return a;
}

void set_active(cs_ctx* c, const std::vector<int>& act) {
  c->cur_act = live(c, act);
  CK(cudaMemcpyAsync(c->A.active, c->cur_act.data(), sizeof(int) * c->cur_act.size(), cudaMemcpyHostToDevice,
                     c->stream));
}

// cloths whose broad phase flagged them as blown up stop here
void note_divergence(cs_ctx* c) {
  for (int i = 0; i < c->A.ni; i++)
    if (c->hst[i].diverged && !c->dead[i]) {
      c->dead[i] = 1;
      c->cloths[c->order[i]]->stats.diverged = 1;
    }
}

void pull_states(cs_ctx* c) {
  c->hst.resize(c->A.ni);
  CK(cudaMemcpyAsync(c->hst.data(), c->A.st, sizeof(InstState) * (size_t)c->A.ni, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
}

// ---- implicit step --------------------------------------------------------------
void assemble(cs_ctx* c) {
  const Arena& A = c->A;
  launch_elements(A, true, true, c->stream);
  launch_slot_reduce(A, c->stream);
  launch_rhs(A, c->stream);
}

// CG on the cloths flagged in cg (others must be inactive for the duration)
void run_cg(cs_ctx* c, const std::vector<int>& cg, double tol, int maxit) {
  const Arena& A = c->A;
  set_active(c, cg);
  int cap = 0;
  bool serial = false;
  for (int i = 0; i < A.ni; i++)
    if (cg[i]) {
      const cs_params& p = c->cloths[c->order[i]]->prm;
      cap = std::max(cap, maxit >= 0 ? maxit : p.maxit);
      serial |= (p.flags & CS_FLAG_EXACT_DOTS) != 0;
    }
  launch_cg_init(A, tol, maxit, c->stream);
  for (int it = 1; it < cap; it++) {
    launch_cg_iteration(A, it, tol, maxit, serial, c->stream);
    if (it % 8 == 0) {
      pull_states(c);
      bool all = true;
      for (int i = 0; i < A.ni; i++)
        if (cg[i] && !c->hst[i].done) all = false;
      if (all) break;
    }
  }
}

// Mixed precision: FP64 refinement cycles around FP32 block-Jacobi CG solves
// (inner relative residual eta, at most `cap` iterations per cycle).
void run_mixed(cs_ctx* c, const std::vector<int>& act) {
  const Arena& A = c->A;
  const float eta = c->mx_eta;
  const int cap = c->mx_cap, maxcycles = 12;
  set_active(c, act);
  launch_mx_outer_init(A, c->stream);
  launch_mx_warm_start(A, c->stream);
  for (int cyc = 0; cyc < maxcycles; cyc++) {
    unsigned gave_up = 0;
    if (c->mx_persistent) {
      launch_mx_inner_persistent(A, eta, cap, c->mx_blocks_per_sm, c->mx_threads, c->mx_tail_slices, c->stream);
      CK(cudaMemcpyAsync(&gave_up, A.grid_bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    } else {
      launch_mx_inner_init(A, c->stream);
      for (int it = 1; it <= cap; it++) {
        launch_mx_inner_iteration(A, it, eta, cap, c->stream);
        if (it % 8 == 0) {
          pull_states(c);
          bool all = true;
          for (int i = 0; i < A.ni; i++)
            if (act[i] && !c->hst[i].done && !c->hst[i].idone) all = false;
          if (all) break;
        }
      }
    }
    launch_mx_refine(A, -1.0, maxcycles, c->stream);
    pull_states(c);
    if (gave_up) throw CudaError("mixed inner solve: a grid barrier wait ran out");
    bool all = true;
    for (int i = 0; i < A.ni; i++)
      if (act[i] && !c->hst[i].done) all = false;
    if (all) break;
  }
}

// solves A dx = b for the active cloths with each cloth's own solver
void solve(cs_ctx* c, const std::vector<int>& act) {
  const Arena& A = c->A;
  if (c->precision == CS_PREC_MIXED) {
    run_mixed(c, act);
    return;
  }
  std::vector<int> ilu, cg(A.ni, 0);
  bool any_cg = false;
  for (int i = 0; i < A.ni; i++) {
    if (!act[i]) continue;
    if (c->solver[i] == CS_SOLVER_CG) {
      cg[i] = 1;
      any_cg = true;
    } else {
      ilu.push_back(i);
    }
  }
  if (!ilu.empty()) {
    CK(cudaMemcpyAsync(c->d_list, ilu.data(), sizeof(int) * ilu.size(), cudaMemcpyHostToDevice, c->stream));
    launch_ilu_factor(A, c->d_list, (int)ilu.size(), c->stream);
    launch_pcg(A, c->d_list, (int)ilu.size(), -1.0, -1, c->stream);
  }
  if (any_cg) run_cg(c, cg, -1.0, -1);
  set_active(c, act);
}

void implicit(cs_ctx* c, const std::vector<int>& act) {
  set_active(c, act);
  assemble(c);
  solve(c, act);
  launch_finish_implicit(c->A, c->stream);
}

// ---- contacts ---------------------------------------------------------------------
// largest pair / candidate buffers (2 GB of leaf pairs, 4 GB of candidates): a
// detection that needs more fails with CS_ERR_CAPACITY instead of growing on
constexpr long long kMaxPairs = 1LL << 28;
constexpr long long kMaxCandidates = 1LL << 25;

// FNV-1a over the 32-bit words of an ordered contact list (5 words a contact,
// cloth-local vertex ids), the digest of the contact log
unsigned long long contact_digest(const int* ce, long long n) {
  unsigned long long d = 14695981039346656037ULL;
  for (long long i = 0; i < 5 * n; i++) {
    d ^= (unsigned long long)(unsigned)ce[i];
    d *= 1099511628211ULL;
  }
  return d;
}

// appends the last detection's ordered contact list of every active cloth to
// the contact log (host copies: a test facility, off by default)
void log_detection(cs_ctx* c, int ccd, int total) {
  const int ni = c->A.ni;
  std::vector<int> lo(ni);
  std::vector<int> ce(5 * (size_t)std::max(total, 1));
  CK(cudaMemcpyAsync(lo.data(), c->C.ce_inst_lo, sizeof(int) * ni, cudaMemcpyDeviceToHost, c->stream));
  if (total > 0)
    CK(cudaMemcpyAsync(ce.data(), c->C.ce, sizeof(int) * 5 * (size_t)total, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < ni; i++) {
    if (i >= (int)c->cur_act.size() || !c->cur_act[i]) continue;
    const int n = c->hst[i].n_contacts, vo = c->voff[i];
    std::vector<int> loc(5 * (size_t)std::max(n, 1));
    for (int e = 0; e < n; e++) {
      loc[5 * e] = ce[5 * ((size_t)lo[i] + e)];
      for (int k = 1; k < 5; k++) loc[5 * e + k] = ce[5 * ((size_t)lo[i] + e) + k] - vo;
    }
    c->clog[c->order[i]].push_back({ccd, n, contact_digest(loc.data(), n)});
  }
}

// detection for the active cloths; returns the total number of contacts and
// leaves per-cloth counts in c->hst.  incremental (CCD only): the previous
// detection's candidates are kept for pairs without a dirty triangle and only
// leaf pairs with a dirty triangle are tested again; the result is the same as
// a full detection because a test depends only on x and its vertices' velocities.
int detect(cs_ctx* c, int ccd, const double* xs, const double* vs, double delta_override,
           bool incremental = false) {
  cudaStream_t s = c->stream;
  launch_refit(c->A, ccd, xs, vs, delta_override, s);
  int cnt[4];
  if (incremental && ccd) {
    CK(cudaMemsetAsync(c->C.counters, 0, sizeof(int), s));
    CK(cudaMemsetAsync(c->C.counters + 3, 0, sizeof(int), s));
    launch_keep_clean_candidates(c->A, c->C, c->last_ncand, s);
    launch_traverse_dirty(c->A, c->C, s);
    CK(cudaMemcpyAsync(cnt, c->C.counters, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    bool ok = !cnt[3];
    if (ok) {
      launch_narrow(c->A, c->C, ccd, xs, vs, delta_override, cnt[0], s);
      CK(cudaMemcpyAsync(cnt, c->C.counters, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      ok = !cnt[3];
    }
    if (ok) {
      const int ncand = cnt[1];
      c->max_ncand = std::max<long long>(c->max_ncand, ncand);
      sort_dedupe(c->A, c->C, ncand, s);
      CK(cudaGetLastError());
      int total = 0;
      CK(cudaMemcpyAsync(&total, c->C.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
      pull_states(c);
      note_divergence(c);
      prof_count("pairs", cnt[0]);
      prof_count("candidates", ncand);
      prof_count("contacts", total);
      prof_count("detections", 1);
      c->last_ncand = ncand;
      c->last_nce = total;
      if (c->log_on) log_detection(c, ccd, total);
      return total;
    }
    // a buffer overflowed: fall back to a full detection (which grows the buffers)
  }
  for (int attempt = 0;; attempt++) {
    CK(cudaMemsetAsync(c->C.counters, 0, sizeof(int) * 4, s));
    launch_traverse(c->A, c->C, s);
    CK(cudaMemcpyAsync(cnt, c->C.counters, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!cnt[3]) break;
    // with the overflow flag set, a count below the capacity means the counter wrapped
    const long long need = (long long)(unsigned)cnt[0];
    if (attempt > 4 || need > kMaxPairs || need < c->C.pair_cap)
      throw CapacityError("broad phase: more than " + std::to_string(kMaxPairs) +
                          " overlapping leaf pairs (boxes of a cloth overlap almost everywhere)");
    alloc_contacts(c, (int)std::min(2 * need + 4096, kMaxPairs), c->C.cand_cap);
  }
  const int npairs = cnt[0];
  for (int attempt = 0;; attempt++) {
    CK(cudaMemsetAsync(c->C.counters + 1, 0, sizeof(int) * 3, s));
    launch_narrow(c->A, c->C, ccd, xs, vs, delta_override, npairs, s);
    int all[8];
    CK(cudaMemcpyAsync(all, c->C.counters, sizeof(int) * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::memcpy(cnt, all, sizeof(int) * 4);
    if (!cnt[3]) break;
    // candidates or a test queue overflowed (a queue holds at most 15 tests per pair)
    const long long need = (long long)(unsigned)cnt[1];
    const long long nfv = (long long)(unsigned)all[6], nee = (long long)(unsigned)all[7];
    const bool over_c = need >= c->C.cand_cap, over_fv = nfv > c->C.q_cap[0], over_ee = nee > c->C.q_cap[1];
    if (attempt > 4 || need > kMaxCandidates || nfv > 6LL * npairs || nee > 9LL * npairs ||
        !(over_c || over_fv || over_ee))
      throw CapacityError("narrow phase: more than " + std::to_string(kMaxCandidates) + " contact candidates");
    const int pairs_keep = c->C.pair_cap;
    const long long qmax = 0x7fffffffLL;
    const int q_fv = over_fv ? (int)std::min({2 * nfv + 4096, 6LL * npairs + 4096, qmax}) : c->C.q_cap[0];
    const int q_ee = over_ee ? (int)std::min({2 * nee + 4096, 9LL * npairs + 4096, qmax}) : c->C.q_cap[1];
    // the pair list must survive the regrow: recompute it after growing
    alloc_contacts(c, pairs_keep, over_c ? (int)std::min(2 * need + 4096, kMaxCandidates) : c->C.cand_cap, q_fv,
                   q_ee);
    CK(cudaMemsetAsync(c->C.counters, 0, sizeof(int) * 4, s));
    launch_traverse(c->A, c->C, s);
  }
  const int ncand = cnt[1];
  c->max_ncand = std::max<long long>(c->max_ncand, ncand);
  sort_dedupe(c->A, c->C, ncand, s);
  CK(cudaGetLastError());
  int total = 0;
  CK(cudaMemcpyAsync(&total, c->C.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  pull_states(c);
  note_divergence(c);
  prof_count("pairs", npairs);
  prof_count("candidates", ncand);
  prof_count("contacts", total);
  prof_count("detections", 1);
  c->last_ncand = ncand;
  c->last_nce = total;
  if (c->log_on) log_detection(c, ccd, total);
  return total;
}

void impulses(cs_ctx* c, int ccd, const double* xs, double* vs) {
  launch_impulses(c->A, c->C, ccd, xs, vs, c->stream);
}

void drop_dead(const cs_ctx* c, std::vector<int>& phase, std::vector<int>& applied) {
  for (size_t i = 0; i < phase.size(); i++)
    if (c->dead[i]) phase[i] = applied[i] = 0;
}

// GetIntermidiateVelocityContactResolved (self_collision_cloth.cpp:355-456) for
// the cloths in act, positions A.x1, velocities A.v in place; returns the
// impulse-applied flag per cloth
std::vector<int> resolve(cs_ctx* c, const std::vector<int>& act) {
  const Arena& A = c->A;
  const int ni = A.ni;
  std::vector<int> applied(ni, 0), phase = act;
  for (int i = 0; i < ni; i++)
    if (act[i]) {
      if (c->log_on) c->clog[c->order[i]].clear();
      cs_stats& st = c->cloths[c->order[i]]->stats;
      const int it = st.solver_iterations, sing = st.ilu_singular;
      const double conv = st.solver_conv;
      std::memset(&st, 0, sizeof(st));
      st.solver_iterations = it;
      st.ilu_singular = sing;
      st.solver_conv = conv;
    }
  set_active(c, phase);
  detect(c, 0, A.x1, nullptr, -1.0);
  drop_dead(c, phase, applied);
  for (int i = 0; i < ni; i++)
    if (act[i]) {
      c->cloths[c->order[i]]->stats.n_prx = c->hst[i].n_contacts;
      applied[i] = c->hst[i].n_contacts > 0;
    }
  impulses(c, 0, A.x1, A.v);
  for (int it = 0; it < 5; it++) {
    bool any = false;
    for (int i = 0; i < ni; i++) any |= phase[i] != 0;
    if (!any) break;
    set_active(c, phase);
    if (it > 0) launch_mark_dirty(A, c->C, c->last_nce, false, c->stream);
    detect(c, 1, A.x1, A.v, -1.0, it > 0);
    drop_dead(c, phase, applied);
    for (int i = 0; i < ni; i++) {
      if (!phase[i]) continue;
      cs_stats& st = c->cloths[c->order[i]]->stats;
      st.n_ccd[it] = c->hst[i].n_contacts;
      st.n_ccd_passes = it + 1;
      if (c->hst[i].n_contacts == 0)
        phase[i] = 0;
      else
        applied[i] = 1;
    }
    set_active(c, phase);
    impulses(c, 1, A.x1, A.v);
  }
  bool any = false;
  for (int i = 0; i < ni; i++) any |= phase[i] != 0;
  if (any) {
    set_active(c, phase);
    CK(cudaMemcpyAsync(A.v0, A.v, sizeof(double) * 3 * (size_t)A.nv, cudaMemcpyDeviceToDevice, c->stream));
    launch_riz_reset(A, c->stream);
    for (int it = 0; it < 100; it++) {
      bool more = false;
      for (int i = 0; i < ni; i++) more |= phase[i] != 0;
      if (!more) break;
      set_active(c, phase);
      // velocities changed at the last pass's contacts (first pass: the fifth
      // CCD impulses) or, after a zone pass, at the zone vertices
      launch_mark_dirty(A, c->C, c->last_nce, it > 0, c->stream);
      detect(c, 1, A.x1, A.v, -1.0, true);
      drop_dead(c, phase, applied);
      launch_riz_count(A, c->stream);
      pull_states(c);
      int nce = 0;
      CK(cudaMemcpyAsync(&nce, c->C.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      for (int i = 0; i < ni; i++) {
        if (!phase[i]) continue;
        cs_stats& st = c->cloths[c->order[i]]->stats;
        const int n = c->hst[i].n_contacts;
        st.n_riz_passes++;
        st.n_riz_last = n;
        st.n_riz_total += n;
        st.riz_nodes = c->hst[i].riz_nodes;
        if (n == 0) phase[i] = 0;
      }
      set_active(c, phase);
      bool work = false;
      for (int i = 0; i < ni; i++) work |= phase[i] != 0;
      if (!work) break;
      launch_riz_add(A, c->C, nce, c->stream);
      c->max_zone = std::max<long long>(c->max_zone, riz_apply(A, c->C, A.x1, A.v, A.v0, c->stream));
    }
  }
  for (int i = 0; i < ni; i++)
    if (act[i]) c->cloths[c->order[i]]->stats.impulse_applied = applied[i];
  set_active(c, act);
  return applied;
}

void update_velocity(cs_ctx* c, const std::vector<int>& act) {
  set_active(c, act);
  launch_elements(c->A, false, true, c->stream);
  launch_update_velocity(c->A, c->stream);
}

// one frame for the cloths in act (StepTime, self_contact_sparse/main.cpp:213-263)
// whether the next frame can run as a captured graph: not while per-kernel
// timing or the contact log need the host between launches, nor on the
// launch-per-iteration mixed solve
bool graph_ok(const cs_ctx* c, const std::vector<int>& act) {
  if (!c->graph_mode || c->A.ni == 0 || prof_enabled() || c->log_on) return false;
  if (c->precision == CS_PREC_MIXED && !c->mx_persistent) return false;
  for (int a : act)
    if (a) return true;
  return false;
}

void frame(cs_ctx* c, const std::vector<int>& act_in) {
  const Arena& A = c->A;
  const std::vector<int> act = live(c, act_in);
  if (graph_ok(c, act) && graph_frame(c, act)) return;
  c->host_frames++;
  CK(cudaMemcpyAsync(A.x1, A.x, sizeof(double) * 3 * (size_t)A.nv, cudaMemcpyDeviceToDevice, c->stream));
  implicit(c, act);
  pull_states(c);
  note_divergence(c);
  for (int i = 0; i < A.ni; i++)
    if (act[i]) {
      cs_stats& st = c->cloths[c->order[i]]->stats;
      st.solver_iterations = c->hst[i].solver_iterations;
      st.solver_conv = c->hst[i].solver_conv;
      st.ilu_singular = c->solver[i] == CS_SOLVER_ILU_PCG ? c->hst[i].ilu_singular : 0;
    }
  std::vector<int> applied = resolve(c, live(c, act));
  bool any = false;
  for (int i = 0; i < A.ni; i++) any |= applied[i] != 0;
  if (any) {
    set_active(c, applied);
    launch_reintegrate(A, c->stream);
    update_velocity(c, applied);
  }
  set_active(c, act);
}

std::vector<int> only(cs_ctx* c, int slot) {
  std::vector<int> a(c->A.ni, 0);
  a[slot] = 1;
  return a;
}

void up(cs_ctx* c, double* dst, const double* src, size_t n) {
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
}
void down(cs_ctx* c, double* dst, const double* src, size_t n) {
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
}

int status_of(const std::exception& e, std::string* msg) {
  if (msg) *msg = e.what();
  if (dynamic_cast<const CapacityError*>(&e)) return CS_ERR_CAPACITY;
  if (dynamic_cast<const CudaError*>(&e))
    return std::string(e.what()).find("out of memory") != std::string::npos ? CS_ERR_OOM : CS_ERR_CUDA;
  return CS_ERR_ARG;
}

template <typename F>
int guarded(cs_ctx* c, F&& f) {
  if (!c) return CS_ERR_ARG;
  try {
    f();
    return CS_OK;
  } catch (const std::exception& e) {
    return status_of(e, &c->err);
  }
}

std::unique_ptr<Cloth> make_cloth(int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                                  const int* quad, const cs_params* prm) {
  if (np <= 0 || nt <= 0 || nq < 0 || !X0 || !tri || (nq > 0 && !quad) || !prm)
    throw ArgError("bad sizes or null arrays");
  if (prm->solver_kind != CS_SOLVER_ILU_PCG && prm->solver_kind != CS_SOLVER_CG) throw ArgError("unknown solver");
  if (prm->obstacle_kind < 0 || prm->obstacle_kind > 3) throw ArgError("unknown obstacle");
  for (int k = 0; k < 3 * nt; k++)
    if (tri[k] < 0 || tri[k] >= np) throw ArgError("triangle index out of range");
  for (int k = 0; k < 4 * nq; k++)
    if (quad[k] < 0 || quad[k] >= np) throw ArgError("stencil index out of range");
  std::unique_ptr<Cloth> cl(new Cloth());
  std::vector<int> bcv(np, 0);
  if (bc) bcv.assign(bc, bc + np);
  build_topology(cl->topo, np, X0, bcv.data(), nt, tri, nq, quad, prm->solver_kind == CS_SOLVER_ILU_PCG);
  cl->prm = *prm;
  cl->x.assign(X0, X0 + 3 * (size_t)np);
  cl->v.assign(3 * (size_t)np, 0.0);
  return cl;
}

size_t cloth_device_bytes(const ClothTopo& t) {
  const size_t np = t.np, nt = t.nt, nq = t.nq, nb = t.nb, nn = t.nnode;
  const size_t slots = t.slot_src.size() + t.grad_src.size() + 2 * (nb + 2 * np);
  size_t b = 0;
  b += np * (5 * 24 + 4 * 2);                  // X0 x v x1 v0, bc vinst
  b += nt * (16 + 81 * 8 + 9 * 8);             // tri tinst, element blocks and gradients
  b += nq * (20 + 4 * 8 + 8 + 12 * 8);         // quad qinst, bending factors, gradients
  b += (np + 1) * 8 + nb * 8;                  // row_ptr dia_split, col_idx blk_row
  b += slots * 4;                              // slot and gradient source lists
  b += (nb + np) * 9 * 8 * 2;                  // matrix and ILU factor values
  b += np * 5 * 24;                            // b r p z dx
  b += (t.lev_rows.size() + t.blev_rows.size() + t.lev_ptr.size() + t.blev_ptr.size() + t.fac_ops.size() +
        np + 1) * 4 + np * 4;                  // ILU schedule, singular flags
  b += nn * (7 * 4 + 4 + 48 + 24 + 4) + nt * 4; // BVH arrays, counters, boxes (FP64 + FP32), tri_leaf
  b += np * (24 + 3 * 4) + t.edge_uv.size() * 4;  // vertex boxes (FP32), dirty / zone flags, edges
  const size_t sell = ((np + 31) / 32) * 32 * 16;  // SELL entries, padded to the slice width
  b += sell * (36 + 4) + (nb + np) * 8;        // FP32 values, columns, SELL positions
  b += np * (36 + 10 * 16);                    // FP32 diagonal inverse and the 10 solver vectors (16 B each)
  // pairs, the test queues and the queues of the certificates' piece stage
  // (face-vertex half a pair capacity, edge-edge two), and the candidate buffers
  b += (16 * nt + 4096) * 8 * 6 + (4 * nt + 4096) * 192;
  b += np * (2 * 4 + 2 * 8 + 72);              // vertex marks, zone keys and sums
  b += np * 48;                                // FP32 hi/lo positions and displacements
  return b + (1 << 16);
}

Cloth& cloth_at(cs_ctx* c, int id) {
  auto it = c->cloths.find(id);
  if (it == c->cloths.end()) throw ArgError("unknown cloth id " + std::to_string(id));
  return *it->second;
}

void ensure(cs_ctx* c) {
  if (c->dirty) rebuild(c);
  CK(cudaSetDevice(c->device));
}

}  // namespace host
}  // namespace cs

using namespace cs::host;

extern "C" {

int cs_create(int device, int precision, cs_ctx** out) {
  if (!out) return CS_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CS_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return CS_ERR_ARG;
  if (precision != CS_PREC_FP64 && precision != CS_PREC_MIXED) return CS_ERR_ARG;
  cs_ctx* c = new cs_ctx();
  c->device = device;
  c->precision = precision;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return CS_ERR_CUDA;
  }
  c->launches0 = g_launches;
  if (const char* e = std::getenv("CLOTHGPU_MX_PERSISTENT")) c->mx_persistent = std::atoi(e) != 0;
  if (const char* e = std::getenv("CLOTHGPU_MX_BLOCKS_PER_SM")) c->mx_blocks_per_sm = std::atoi(e);
  if (const char* e = std::getenv("CLOTHGPU_MX_ETA")) c->mx_eta = (float)std::atof(e);
  if (const char* e = std::getenv("CLOTHGPU_MX_ETA_BIG")) c->mx_eta_big = (float)std::atof(e);
  if (const char* e = std::getenv("CLOTHGPU_MX_THREADS")) c->mx_threads = std::atoi(e);
  if (const char* e = std::getenv("CLOTHGPU_MX_CAP")) c->mx_cap = std::atoi(e);
  if (const char* e = std::getenv("CLOTHGPU_MX_TAIL_SLICES")) c->mx_tail_slices = std::atoi(e);
  if (const char* e = std::getenv("CLOTHGPU_NARROW_REGS")) c->narrow_regs = std::atoi(e) == 128 ? 128 : 0;
  // contexts made by the library itself (the serving loop) take the frame mode from here
  if (const char* e = std::getenv("CLOTHGPU_FRAME_MODE")) c->graph_mode = std::strcmp(e, "host") != 0;
  if (const char* e = std::getenv("CLOTHGPU_BAR_SLEEP_NS")) c->bar_sleep_ns = std::max(0, std::atoi(e));
  if (const char* e = std::getenv("CLOTHGPU_IMPULSE_CLUSTER")) c->impulse_cluster = std::atoi(e) == 8 ? 8 : 1;
  // failure-detection tests: a short barrier time-out, and a barrier that
  // block 0 never reaches (every wait then runs out and the frame fails with
  // CS_ERR_CUDA, the context staying usable)
  if (const char* e = std::getenv("CLOTHGPU_BAR_TIMEOUT_NS")) c->bar_timeout_ns = std::max(1000LL, std::atoll(e));
  if (const char* e = std::getenv("CLOTHGPU_BAR_HOLD")) c->bar_hold = std::atoi(e) != 0;
  c->A.narrow_regs = c->narrow_regs;
  c->A.bar_sleep_ns = c->bar_sleep_ns;
  c->A.impulse_cluster = c->impulse_cluster;
  c->A.mx_eta_big = c->mx_eta_big;
  c->A.bar_timeout_ns = c->bar_timeout_ns;
  c->A.bar_hold = c->bar_hold;
  *out = c;
  return CS_OK;
}

void cs_destroy(cs_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  graph_release(c);
  if (c->gsave) cudaFree(c->gsave);
  for (cudaStream_t g : c->gstream)
    if (g) cudaStreamDestroy(g);
  c->mem.release();
  c->cmem.release();
  cudaStreamDestroy(c->stream);
  delete c;
}

const char* cs_last_error(const cs_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* cs_stream(const cs_ctx* c) { return c ? (void*)c->stream : nullptr; }

int cs_set_precision(cs_ctx* c, int precision) {
  return guarded(c, [&] {
    if (precision != CS_PREC_FP64 && precision != CS_PREC_MIXED) throw ArgError("unknown precision");
    graph_release(c);
    c->precision = precision;
  });
}

int cs_synchronize(cs_ctx* c) {
  return guarded(c, [&] { CK(cudaStreamSynchronize(c->stream)); });
}

int cs_add_cloth(cs_ctx* c, int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                 const int* quad, const cs_params* prm, int* id_out) {
  return guarded(c, [&] {
    std::unique_ptr<Cloth> cl;
    try {
      cl = make_cloth(np, X0, bc, nt, tri, nq, quad, prm);
    } catch (const ArgError& e) {
      throw ArgError(std::string("cs_add_cloth: ") + e.what());
    }
    save_states(c);
    cl->id = c->next_id++;
    c->order.push_back(cl->id);
    if (id_out) *id_out = cl->id;
    c->cloths[cl->id] = std::move(cl);
    c->dirty = true;
  });
}

int cs_remove_cloth(cs_ctx* c, int id) {
  return guarded(c, [&] {
    cloth_at(c, id);
    save_states(c);
    c->order.erase(std::find(c->order.begin(), c->order.end(), id));
    c->cloths.erase(id);
    c->dirty = true;
  });
}

int cs_num_cloths(const cs_ctx* c) { return c ? (int)c->order.size() : 0; }

int cs_set_params(cs_ctx* c, int id, const cs_params* prm) {
  return guarded(c, [&] {
    if (!prm) throw ArgError("null params");
    Cloth& cl = cloth_at(c, id);
    graph_release(c);  // solver lists and caps are part of the graph
    if (prm->solver_kind != cl.prm.solver_kind) {
      // the ILU schedule is part of the topology
      save_states(c);
      build_topology(cl.topo, cl.topo.np, cl.topo.X0.data(), cl.topo.bc.data(), cl.topo.nt, cl.topo.tri.data(),
                     cl.topo.nq, cl.topo.quad.data(), prm->solver_kind == CS_SOLVER_ILU_PCG);
      cl.prm = *prm;
      c->dirty = true;
      return;
    }
    cl.prm = *prm;
    if (!c->dirty) {
      const DevParams d = to_dev(*prm);
      CK(cudaMemcpyAsync(c->A.prm + slot_of(c, id), &d, sizeof(d), cudaMemcpyHostToDevice, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      launch_quad_factors(c->A, c->stream);  // bending stiffness may have changed
    }
  });
}

int cs_set_state(cs_ctx* c, int id, const double* x, const double* v) {
  return guarded(c, [&] {
    Cloth& cl = cloth_at(c, id);
    if (c->dirty) {
      if (x) cl.x.assign(x, x + cl.x.size());
      if (v) cl.v.assign(v, v + cl.v.size());
      return;
    }
    const int i = slot_of(c, id);
    if (x) up(c, c->A.x + 3 * (size_t)c->voff[i], x, cl.x.size());
    if (v) up(c, c->A.v + 3 * (size_t)c->voff[i], v, cl.v.size());
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_get_state(cs_ctx* c, int id, double* x, double* v) {
  return guarded(c, [&] {
    Cloth& cl = cloth_at(c, id);
    if (c->dirty) {
      if (x) std::memcpy(x, cl.x.data(), sizeof(double) * cl.x.size());
      if (v) std::memcpy(v, cl.v.data(), sizeof(double) * cl.v.size());
      return;
    }
    const int i = slot_of(c, id);
    if (x) down(c, x, c->A.x + 3 * (size_t)c->voff[i], cl.x.size());
    if (v) down(c, v, c->A.v + 3 * (size_t)c->voff[i], cl.v.size());
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_get_stats(cs_ctx* c, int id, cs_stats* st) {
  return guarded(c, [&] {
    if (!st) throw ArgError("null stats");
    *st = cloth_at(c, id).stats;
  });
}

int cs_step(cs_ctx* c, int nsteps) {
  return guarded(c, [&] {
    if (nsteps < 0) throw ArgError("negative step count");
    ensure(c);
    if (c->A.ni == 0) return;
    std::vector<int> all(c->A.ni, 1);
    for (int k = 0; k < nsteps; k++) frame(c, all);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
  });
}

int cs_implicit_step(cs_ctx* c, int id, double* x, double* v, cs_stats* st) {
  return guarded(c, [&] {
    if (!x || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t n = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.x + 3 * (size_t)c->voff[i], x, n);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, n);
    implicit(c, only(c, i));
    pull_states(c);
    down(c, x, c->A.x + 3 * (size_t)c->voff[i], n);
    down(c, v, c->A.v + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
    if (st) {
      std::memset(st, 0, sizeof(*st));
      st->solver_iterations = c->hst[i].solver_iterations;
      st->solver_conv = c->hst[i].solver_conv;
      st->ilu_singular = c->solver[i] == CS_SOLVER_ILU_PCG ? c->hst[i].ilu_singular : 0;
    }
  });
}

int cs_resolve_contacts(cs_ctx* c, int id, const double* x1, double* v, cs_stats* st) {
  return guarded(c, [&] {
    if (!x1 || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t n = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x1, n);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, n);
    resolve(c, only(c, i));
    down(c, v, c->A.v + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
    if (st) *st = c->cloths[id]->stats;
  });
}

int cs_update_velocity(cs_ctx* c, int id, const double* x, double* v) {
  return guarded(c, [&] {
    if (!x || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t n = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.x + 3 * (size_t)c->voff[i], x, n);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, n);
    update_velocity(c, only(c, i));
    down(c, v, c->A.v + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_assemble(cs_ctx* c, int id, const double* x, const double* v, double* vdia, double* vcrs, double* b) {
  return guarded(c, [&] {
    if (!x || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.x + 3 * (size_t)c->voff[i], x, 3 * (size_t)t.np);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, 3 * (size_t)t.np);
    set_active(c, only(c, i));
    assemble(c);
    if (vdia) down(c, vdia, c->A.vdia + 9 * (size_t)c->voff[i], 9 * (size_t)t.np);
    if (vcrs) down(c, vcrs, c->A.vcrs + 9 * (size_t)c->boff[i], 9 * (size_t)t.nb);
    if (b) down(c, b, c->A.b + 3 * (size_t)c->voff[i], 3 * (size_t)t.np);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_pattern(cs_ctx* c, int id, int* nb, int* row_ptr, int* col_idx) {
  return guarded(c, [&] {
    const ClothTopo& t = cloth_at(c, id).topo;
    if (nb) *nb = t.nb;
    if (row_ptr) std::memcpy(row_ptr, t.row_ptr.data(), sizeof(int) * t.row_ptr.size());
    if (col_idx) std::memcpy(col_idx, t.col_idx.data(), sizeof(int) * t.col_idx.size());
  });
}

int cs_ilu_factor(cs_ctx* c, int id, double* fdia, double* fcrs, int* nsing) {
  return guarded(c, [&] {
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    if (t.lev_ptr.empty()) throw ArgError("cloth was added without the ILU(0) solver");
    CK(cudaMemcpyAsync(c->d_list, &i, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    launch_ilu_factor(c->A, c->d_list, 1, c->stream);
    if (fdia) down(c, fdia, c->A.fdia + 9 * (size_t)c->voff[i], 9 * (size_t)t.np);
    if (fcrs) down(c, fcrs, c->A.fcrs + 9 * (size_t)c->boff[i], 9 * (size_t)t.nb);
    pull_states(c);
    if (nsing) *nsing = c->hst[i].ilu_singular;
  });
}

int cs_solve_pcg(cs_ctx* c, int id, const double* b, double tol, int maxit, double* x, double* conv, int* iter) {
  return guarded(c, [&] {
    if (!b || !x) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    if (t.lev_ptr.empty()) throw ArgError("cloth was added without the ILU(0) solver");
    up(c, c->A.b + 3 * (size_t)c->voff[i], b, 3 * (size_t)t.np);
    CK(cudaMemcpyAsync(c->d_list, &i, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    launch_pcg(c->A, c->d_list, 1, tol, maxit, c->stream);
    down(c, x, c->A.dx + 3 * (size_t)c->voff[i], 3 * (size_t)t.np);
    pull_states(c);
    if (conv) *conv = c->hst[i].solver_conv;
    if (iter) *iter = c->hst[i].solver_iterations;
  });
}

int cs_solve_cg(cs_ctx* c, int id, const double* b, double tol, int maxit, double* x, double* conv, int* iter) {
  return guarded(c, [&] {
    if (!b || !x) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.b + 3 * (size_t)c->voff[i], b, 3 * (size_t)t.np);
    run_cg(c, only(c, i), tol, maxit);
    down(c, x, c->A.dx + 3 * (size_t)c->voff[i], 3 * (size_t)t.np);
    pull_states(c);
    if (conv) *conv = c->hst[i].solver_conv;
    if (iter) *iter = c->hst[i].solver_iterations;
  });
}

int cs_spmv(cs_ctx* c, int id, const double* x, double* y) {
  return guarded(c, [&] {
    if (!x || !y) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t n = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.p + 3 * (size_t)c->voff[i], x, n);
    CK(cudaMemsetAsync(c->A.z, 0, sizeof(double) * 3 * (size_t)c->A.nv, c->stream));
    launch_spmv(c->A, c->A.p, c->A.z, c->stream);
    down(c, y, c->A.z + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_last_residual(cs_ctx* c, int id, double* r) {
  return guarded(c, [&] {
    if (!r) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    down(c, r, c->A.r + 3 * (size_t)c->voff[i], 3 * (size_t)c->cloths[id]->topo.np);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_set_matrix(cs_ctx* c, int id, const double* vdia, const double* vcrs) {
  return guarded(c, [&] {
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    if (vdia) up(c, c->A.vdia + 9 * (size_t)c->voff[i], vdia, 9 * (size_t)t.np);
    if (vcrs) up(c, c->A.vcrs + 9 * (size_t)c->boff[i], vcrs, 9 * (size_t)t.nb);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_matvec(cs_ctx* c, int id, double alpha, const double* x, double beta, double* y) {
  return guarded(c, [&] {
    if (!x || !y) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t n = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.p + 3 * (size_t)c->voff[i], x, n);
    up(c, c->A.z + 3 * (size_t)c->voff[i], y, n);
    launch_matvec(c->A, c->voff[i], c->voff[i + 1], alpha, c->A.p, beta, c->A.z, c->stream);
    down(c, y, c->A.z + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_ilu_solve(cs_ctx* c, int id, double* vec) {
  return guarded(c, [&] {
    if (!vec) throw ArgError("null vector");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    if (t.lev_ptr.empty()) throw ArgError("cloth was added without the ILU(0) solver");
    const size_t n = 3 * (size_t)t.np;
    up(c, c->A.z + 3 * (size_t)c->voff[i], vec, n);
    launch_ilu_solve(c->A, i, c->A.z, c->stream);
    down(c, vec, c->A.z + 3 * (size_t)c->voff[i], n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_bvh_nodes(cs_ctx* c, int id, int* nnode, int* nodes) {
  return guarded(c, [&] {
    const ClothTopo& t = cloth_at(c, id).topo;
    if (nnode) *nnode = t.nnode;
    if (nodes) std::memcpy(nodes, t.node.data(), sizeof(int) * t.node.size());
  });
}

static void boxes_out(cs_ctx* c, int i, int nnode, double* boxes) {
  std::vector<Box> hb(nnode);
  CK(cudaMemcpyAsync(hb.data(), c->A.box + c->noff[i], sizeof(Box) * nnode, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int n = 0; n < nnode; n++) {
    for (int k = 0; k < 3; k++) {
      boxes[7 * n + 2 * k] = hb[n].lo[k];
      boxes[7 * n + 2 * k + 1] = hb[n].hi[k];
    }
    boxes[7 * n + 6] = hb[n].full ? 1.0 : 0.0;
  }
}

int cs_get_boxes(cs_ctx* c, int id, double* boxes) {
  return guarded(c, [&] {
    if (!boxes) throw ArgError("null boxes");
    ensure(c);
    boxes_out(c, slot_of(c, id), c->cloths[id]->topo.nnode, boxes);
  });
}

int cs_refit_prx(cs_ctx* c, int id, const double* x, double delta, double* boxes) {
  return guarded(c, [&] {
    if (!x) throw ArgError("null positions");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, 3 * (size_t)t.np);
    set_active(c, only(c, i));
    launch_refit(c->A, 0, c->A.x1, nullptr, delta, c->stream);
    if (boxes) boxes_out(c, i, t.nnode, boxes);
    CK(cudaStreamSynchronize(c->stream));
  });
}

// runs f with the cloth's dt replaced (the CCD stages take dt as an argument)
extern "C++" template <typename F>
void with_dt(cs_ctx* c, int i, int id, double dt, F&& f) {
  cs_params p = c->cloths[id]->prm;
  p.dt = dt;
  DevParams d = to_dev(p), d0 = to_dev(c->cloths[id]->prm);
  CK(cudaMemcpyAsync(c->A.prm + i, &d, sizeof(d), cudaMemcpyHostToDevice, c->stream));
  f();
  CK(cudaMemcpyAsync(c->A.prm + i, &d0, sizeof(d0), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
}

int cs_refit_ccd(cs_ctx* c, int id, const double* x, const double* v, double dt, double* boxes) {
  return guarded(c, [&] {
    if (!x || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, 3 * (size_t)t.np);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, 3 * (size_t)t.np);
    set_active(c, only(c, i));
    with_dt(c, i, id, dt, [&] { launch_refit(c->A, 1, c->A.x1, c->A.v, -1.0, c->stream); });
    if (boxes) boxes_out(c, i, t.nnode, boxes);
  });
}

static void contacts_out(cs_ctx* c, int i, int total, int* out, int cap, int* n) {
  const int cnt = c->hst[i].n_contacts;
  if (n) *n = cnt;
  if (!out) return;
  int lo = 0;
  CK(cudaMemcpyAsync(&lo, c->C.ce_inst_lo + i, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const int m = std::min(cnt, cap);
  std::vector<int> h(5 * (size_t)std::max(m, 1));
  if (m > 0)
    CK(cudaMemcpyAsync(h.data(), c->C.ce + 5 * (size_t)lo, sizeof(int) * 5 * (size_t)m, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const int vo = c->voff[i];
  for (int e = 0; e < m; e++) {
    out[5 * e] = h[5 * e];
    for (int k = 1; k < 5; k++) out[5 * e + k] = h[5 * e + k] - vo;
  }
  (void)total;
  if (cnt > cap) throw CapacityError("contact output buffer too small");
}

int cs_contacts_prx(cs_ctx* c, int id, const double* x, double delta, int* out, int cap, int* n) {
  return guarded(c, [&] {
    if (!x) throw ArgError("null positions");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, 3 * (size_t)t.np);
    set_active(c, only(c, i));
    const int total = detect(c, 0, c->A.x1, nullptr, delta);
    contacts_out(c, i, total, out, cap, n);
  });
}

int cs_contacts_ccd(cs_ctx* c, int id, const double* x, const double* v, double dt, double delta, int* out, int cap,
                    int* n) {
  return guarded(c, [&] {
    if (!x || !v) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const ClothTopo& t = c->cloths[id]->topo;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, 3 * (size_t)t.np);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, 3 * (size_t)t.np);
    set_active(c, only(c, i));
    int total = 0;
    with_dt(c, i, id, dt, [&] { total = detect(c, 1, c->A.x1, c->A.v, delta); });
    contacts_out(c, i, total, out, cap, n);
  });
}

// uploads a host contact list (cloth-local ids) as the cloth's contact segment
static void contacts_in(cs_ctx* c, int i, const int* ce, int n) {
  if (n > c->C.ce_cap) alloc_contacts(c, c->C.pair_cap, n + 4096);
  std::vector<int> h(5 * (size_t)std::max(n, 1));
  const int vo = c->voff[i];
  for (int e = 0; e < n; e++) {
    h[5 * e] = ce[5 * e];
    for (int k = 1; k < 5; k++) h[5 * e + k] = ce[5 * e + k] + vo;
  }
  if (n > 0) CK(cudaMemcpyAsync(c->C.ce, h.data(), sizeof(int) * 5 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  std::vector<int> lo(c->A.ni, 0), hi(c->A.ni, 0);
  hi[i] = n;
  CK(cudaMemcpyAsync(c->C.ce_inst_lo, lo.data(), sizeof(int) * lo.size(), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->C.ce_inst_hi, hi.data(), sizeof(int) * hi.size(), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->C.counters + 2, &n, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
}

static int impulse_api(cs_ctx* c, int id, const double* x, double* v, const int* ce, int n, int ccd) {
  return guarded(c, [&] {
    if (!x || !v || (n > 0 && !ce) || n < 0) throw ArgError("bad arguments");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t nd = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, nd);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, nd);
    set_active(c, only(c, i));
    contacts_in(c, i, ce, n);
    impulses(c, ccd, c->A.x1, c->A.v);
    down(c, v, c->A.v + 3 * (size_t)c->voff[i], nd);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_impulse_prx(cs_ctx* c, int id, const double* x, double* v, const int* ce, int n) {
  return impulse_api(c, id, x, v, ce, n, 0);
}
int cs_impulse_ccd(cs_ctx* c, int id, const double* x, double* v, const int* ce, int n) {
  return impulse_api(c, id, x, v, ce, n, 1);
}

int cs_riz_reset(cs_ctx* c, int id) {
  return guarded(c, [&] {
    ensure(c);
    set_active(c, only(c, slot_of(c, id)));
    launch_riz_reset(c->A, c->stream);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_riz_add(cs_ctx* c, int id, const int* ce, int n) {
  return guarded(c, [&] {
    if ((n > 0 && !ce) || n < 0) throw ArgError("bad arguments");
    ensure(c);
    const int i = slot_of(c, id);
    set_active(c, only(c, i));
    contacts_in(c, i, ce, n);
    launch_riz_add(c->A, c->C, n, c->stream);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_riz_zones(cs_ctx* c, int id, int* zone_of, int* nzone) {
  return guarded(c, [&] {
    ensure(c);
    const int i = slot_of(c, id);
    const int np = c->cloths[id]->topo.np;
    set_active(c, only(c, i));
    riz_count_zones(c->A, c->C, c->C.idx_a, c->stream);  // labels into scratch (needs nv ints)
    std::vector<int> lab(c->A.nv);
    CK(cudaMemcpyAsync(lab.data(), c->C.idx_a, sizeof(int) * (size_t)c->A.nv, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::map<int, int> ids;
    for (int v = 0; v < np; v++) {
      const int r = lab[c->voff[i] + v];
      int z = -1;
      if (r >= 0) {
        auto it = ids.find(r);
        if (it == ids.end()) it = ids.emplace(r, (int)ids.size()).first;
        z = it->second;
      }
      if (zone_of) zone_of[v] = z;
    }
    if (nzone) *nzone = (int)ids.size();
  });
}

int cs_riz_apply(cs_ctx* c, int id, const double* x, double* v, const double* v0) {
  return guarded(c, [&] {
    if (!x || !v || !v0) throw ArgError("null state");
    ensure(c);
    const int i = slot_of(c, id);
    const size_t nd = 3 * (size_t)c->cloths[id]->topo.np;
    up(c, c->A.x1 + 3 * (size_t)c->voff[i], x, nd);
    up(c, c->A.v + 3 * (size_t)c->voff[i], v, nd);
    up(c, c->A.v0 + 3 * (size_t)c->voff[i], v0, nd);
    set_active(c, only(c, i));
    riz_apply(c->A, c->C, c->A.x1, c->A.v, c->A.v0, c->stream);
    down(c, v, c->A.v + 3 * (size_t)c->voff[i], nd);
    CK(cudaStreamSynchronize(c->stream));
  });
}

extern "C++" template <typename F>
int element_batch(cs_ctx* c, int n, std::initializer_list<std::pair<const double*, size_t>> ins,
                         std::initializer_list<std::pair<double*, size_t>> outs, F&& launch) {
  return guarded(c, [&] {
    if (n < 0) throw ArgError("negative count");
    if (n == 0) return;
    CK(cudaSetDevice(c->device));
    DevMem tmp;
    std::vector<double*> din, dout;
    try {
      for (auto& p : ins) {
        if (!p.first) throw ArgError("null input");
        double* d = tmp.alloc<double>(p.second * n);
        CK(cudaMemcpyAsync(d, p.first, sizeof(double) * p.second * n, cudaMemcpyHostToDevice, c->stream));
        din.push_back(d);
      }
      for (auto& p : outs) dout.push_back(tmp.alloc<double>(p.second * n));
      launch(din, dout);
      size_t k = 0;
      for (auto& p : outs) {
        if (p.first)
          CK(cudaMemcpyAsync(p.first, dout[k], sizeof(double) * p.second * n, cudaMemcpyDeviceToHost, c->stream));
        k++;
      }
      CK(cudaStreamSynchronize(c->stream));
    } catch (...) {
      cudaStreamSynchronize(c->stream);
      tmp.release();
      throw;
    }
    tmp.release();
  });
}

int cs_element_cst(cs_ctx* c, int n, const double* C, const double* cc, double lambda, double myu, double* W,
                   double* dW, double* ddW) {
  return element_batch(c, n, {{C, 9}, {cc, 9}}, {{W, 1}, {dW, 9}, {ddW, 81}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_element_batch_cst(n, i[0], i[1], lambda, myu, o[0], o[1], o[2], c->stream);
                       });
}

int cs_element_bend(cs_ctx* c, int n, const double* C, const double* cc, double stiff, double* W, double* dW,
                    double* ddW) {
  return element_batch(c, n, {{C, 12}, {cc, 12}}, {{W, 1}, {dW, 12}, {ddW, 144}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_element_batch_bend(n, i[0], i[1], stiff, o[0], o[1], o[2], c->stream);
                       });
}

int cs_element_contact(cs_ctx* c, int n, const double* cc, const cs_params* prm, double* W, double* dW,
                       double* ddW) {
  if (!prm) return CS_ERR_ARG;
  const DevParams d = to_dev(*prm);
  return element_batch(c, n, {{cc, 3}}, {{W, 1}, {dW, 3}, {ddW, 9}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_element_batch_contact(n, i[0], &d, o[0], o[1], o[2], c->stream);
                       });
}

int cs_distance_fv(cs_ctx* c, int n, const double* pts, double* dist, double* w) {
  return element_batch(c, n, {{pts, 12}}, {{dist, 1}, {w, 2}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_distance_fv(n, i[0], o[0], o[1], c->stream);
                       });
}

int cs_distance_ee(cs_ctx* c, int n, const double* pts, double* dist, double* ratio) {
  return element_batch(c, n, {{pts, 12}}, {{dist, 1}, {ratio, 2}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_distance_ee(n, i[0], o[0], o[1], c->stream);
                       });
}

int cs_coplanar_time(cs_ctx* c, int n, const double* s0, const double* e0, double* t) {
  return element_batch(c, n, {{s0, 12}, {e0, 12}}, {{t, 1}},
                       [&](std::vector<double*>& i, std::vector<double*>& o) {
                         launch_coplanar_time(n, i[0], i[1], o[0], c->stream);
                       });
}

namespace {
// launch shapes chosen by cs_autotune, per arena shape and precision
struct TuneKey {
  int ni, nv, nslice, precision;
  bool operator<(const TuneKey& o) const {
    return std::tie(ni, nv, nslice, precision) < std::tie(o.ni, o.nv, o.nslice, o.precision);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, cs_tune_result> g_tune;

void apply_tune(cs_ctx* c, const cs_tune_result& r) {
  c->mx_blocks_per_sm = r.mx_blocks_per_sm;
  c->mx_tail_slices = r.mx_tail_slices;
  c->graph_grid_per_sm = r.graph_grid_per_sm;
  c->narrow_regs = r.narrow_regs;
  c->A.narrow_regs = r.narrow_regs;
  c->bar_sleep_ns = r.bar_sleep_ns;
  c->A.bar_sleep_ns = r.bar_sleep_ns;
  c->impulse_cluster = r.impulse_cluster;
  c->A.impulse_cluster = r.impulse_cluster;
  graph_release(c);
}
}  // namespace

int cs_autotune(cs_ctx* c, int frames, cs_tune_result* out) {
  return guarded(c, [&] {
    ensure(c);
    if (c->A.ni == 0) throw ArgError("no cloths to tune on");
    frames = std::max(1, frames);
    const TuneKey key{c->A.ni, c->A.nv, c->A.nslice, c->precision};
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        apply_tune(c, it->second);
        if (out) {
          *out = it->second;
          out->cached = 1;
        }
        return;
      }
    }
    // the start state, restored after every candidate: frames do not depend on
    // these launch shapes, so tuning leaves the simulation where it was
    const size_t n3 = 3 * (size_t)c->A.nv;
    std::vector<double> x(n3), v(n3);
    down(c, x.data(), c->A.x, n3);
    down(c, v.data(), c->A.v, n3);
    CK(cudaStreamSynchronize(c->stream));
    const std::vector<int> dead = c->dead;
    std::vector<cs_stats> stats;
    for (int id : c->order) stats.push_back(c->cloths[id]->stats);
    const std::vector<int> all(c->A.ni, 1);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int timed = 0;
    auto restore = [&] {
      up(c, c->A.x, x.data(), n3);
      up(c, c->A.v, v.data(), n3);
      CK(cudaStreamSynchronize(c->stream));
      c->dead = dead;
      for (size_t i = 0; i < c->order.size(); i++) c->cloths[c->order[i]]->stats = stats[i];
    };
    auto time_cfg = [&](const cs_tune_result& r) {
      apply_tune(c, r);
      restore();
      if (c->graph_mode && graph_ok(c, live(c, all))) {  // capture is not timed
        try {
          graph_capture(c);
        } catch (const CudaError&) {
          c->graph_mode = false;  // as a graph frame would: host-driven from here on
        }
      }
      CK(cudaEventRecord(e0, c->stream));
      for (int f = 0; f < frames; f++) frame(c, all);
      CK(cudaEventRecord(e1, c->stream));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      timed++;
      return (double)ms / frames;
    };
    cs_tune_result best{};
    best.mx_blocks_per_sm = c->mx_blocks_per_sm > 0 ? c->mx_blocks_per_sm : 6;
    best.mx_tail_slices = c->mx_tail_slices;
    best.graph_grid_per_sm = c->graph_grid_per_sm;
    best.narrow_regs = c->narrow_regs;
    best.bar_sleep_ns = c->bar_sleep_ns;
    best.impulse_cluster = c->impulse_cluster;
    time_cfg(best);  // untimed warm pass: contact buffers grow to these frames' needs
    best.frame_ms = time_cfg(best);
    // coordinate descent over the three shapes
    auto try_values = [&](int cs_tune_result::*field, std::initializer_list<int> values) {
      for (int val : values) {
        if (best.*field == val) continue;
        cs_tune_result r = best;
        r.*field = val;
        const double ms = time_cfg(r);
        if (ms < best.frame_ms) {
          best = r;
          best.frame_ms = ms;
        }
      }
    };
    if (c->precision == CS_PREC_MIXED) {
      try_values(&cs_tune_result::mx_blocks_per_sm, {4, 5, 6});
      try_values(&cs_tune_result::mx_tail_slices, {0, 608, 1216, 2432, 4864});
    }
    if (c->graph_mode) try_values(&cs_tune_result::graph_grid_per_sm, {4, 8, 16});
    try_values(&cs_tune_result::narrow_regs, {0, 128});
    if (c->precision == CS_PREC_MIXED) try_values(&cs_tune_result::bar_sleep_ns, {256, 64, 0});
    try_values(&cs_tune_result::impulse_cluster, {1, 8});
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    best.candidates = timed;
    best.cached = 0;
    apply_tune(c, best);
    restore();
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      g_tune[key] = best;
    }
    if (out) *out = best;
  });
}

int cs_set_frame_mode(cs_ctx* c, int mode) {
  return guarded(c, [&] {
    if (mode != CS_FRAME_HOST && mode != CS_FRAME_GRAPH) throw ArgError("unknown frame mode");
    c->graph_mode = mode == CS_FRAME_GRAPH;
    if (!c->graph_mode) graph_release(c);
  });
}

int cs_frame_counts(cs_ctx* c, long long* graph_frames, long long* host_frames, long long* captures,
                    long long* overflows) {
  return guarded(c, [&] {
    if (graph_frames) *graph_frames = c->g_frames;
    if (host_frames) *host_frames = c->host_frames;
    if (captures) *captures = c->g_captures;
    if (overflows) *overflows = c->g_overflows;
  });
}

int cs_frame_overflows(cs_ctx* c, long long* reasons) {
  if (!reasons) return CS_ERR_ARG;
  return guarded(c, [&] {
    for (int k = 0; k < 4; k++) reasons[k] = c->g_over_reason[k];
  });
}

int cs_contact_log(cs_ctx* c, int enable) {
  return guarded(c, [&] {
    c->log_on = enable != 0;
    c->clog.clear();
  });
}

int cs_contact_log_read(cs_ctx* c, int id, int* kind, int* count, unsigned long long* digest, int cap, int* n) {
  return guarded(c, [&] {
    if (!c->cloths.count(id)) throw ArgError("unknown cloth id");
    const auto it = c->clog.find(id);
    const int m = it == c->clog.end() ? 0 : (int)it->second.size();
    if (n) *n = m;
    for (int e = 0; e < m && e < cap; e++) {
      if (kind) kind[e] = it->second[e].kind;
      if (count) count[e] = it->second[e].count;
      if (digest) digest[e] = it->second[e].digest;
    }
    if (m > cap && (kind || count || digest)) throw CapacityError("contact log longer than cap");
  });
}

long long cs_launch_count(const cs_ctx* c) { return c ? g_launches - c->launches0 : 0; }

int cs_profile(cs_ctx* c, int enable) {
  return guarded(c, [&] {
    ensure(c);
    CK(cudaStreamSynchronize(c->stream));
    prof_reset();
    prof_enable(enable != 0);
    c->A.count_bytes = enable != 0;
    if (c->A.bytes_acc) CK(cudaMemsetAsync(c->A.bytes_acc, 0, 8 * sizeof(unsigned long long), c->stream));
  });
}

int cs_profile_bytes(cs_ctx* c, long long* spmv32, long long* spmv64) {
  return guarded(c, [&] {
    ensure(c);
    unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (c->A.bytes_acc)
      CK(cudaMemcpyAsync(h, c->A.bytes_acc, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (spmv32) *spmv32 = (long long)h[0];
    if (spmv64) *spmv64 = (long long)h[1];
    prof_count("fp64_fv_prx", (long long)h[2]);
    prof_count("fp64_ee_prx", (long long)h[3]);
    prof_count("fp64_fv_ccd", (long long)h[4]);
    prof_count("fp64_ee_ccd", (long long)h[5]);
    prof_count("persist_bytes", (long long)h[6]);
  });
}

int cs_profile_read(cs_ctx* c, const char* kernel, double* total_ms, long long* launches) {
  return guarded(c, [&] {
    if (!kernel) throw ArgError("null kernel name");
    CK(cudaStreamSynchronize(c->stream));
    if (!prof_read(kernel, total_ms, launches)) throw ArgError(std::string("unknown kernel class ") + kernel);
  });
}

int cs_set_states(cs_ctx* c, const double* x, const double* v) {
  return guarded(c, [&] {
    ensure(c);
    const size_t n = 3 * (size_t)c->A.nv;
    if (x) up(c, c->A.x, x, n);
    if (v) up(c, c->A.v, v, n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_get_states(cs_ctx* c, double* x, double* v) {
  return guarded(c, [&] {
    ensure(c);
    const size_t n = 3 * (size_t)c->A.nv;
    if (x) down(c, x, c->A.x, n);
    if (v) down(c, v, c->A.v, n);
    CK(cudaStreamSynchronize(c->stream));
  });
}

int cs_vertex_normals(cs_ctx* c, int id, const double* x, double* normals) {
  return guarded(c, [&] {
    if (!normals) throw ArgError("null normals");
    if (id < 0 && x) throw ArgError("positions are per cloth: pass id >= 0 with x");
    ensure(c);
    const Arena& A = c->A;
    if (A.ni == 0) return;
    // dx is a work vector of the implicit step: free between frames
    if (id >= 0) {
      const int i = slot_of(c, id);
      const size_t n = 3 * (size_t)c->cloths[id]->topo.np, off = 3 * (size_t)c->voff[i];
      if (x) up(c, A.x1 + off, x, n);
      set_active(c, only(c, i));
      launch_vertex_normals(A, x ? A.x1 : A.x, A.dx, c->stream);
      down(c, normals, A.dx + off, n);
    } else {
      set_active(c, std::vector<int>(A.ni, 1));
      launch_vertex_normals(A, A.x, A.dx, c->stream);
      down(c, normals, A.dx, 3 * (size_t)A.nv);
    }
    CK(cudaStreamSynchronize(c->stream));
  });
}

long long cs_num_vertices(const cs_ctx* c) {
  if (!c) return 0;
  long long n = 0;
  for (auto& kv : c->cloths) n += kv.second->topo.np;
  return n;
}

int cs_build_bvh(int np, const double* X, int nt, const int* tri, int* nodes, int cap, int* nnode) {
  if (np <= 0 || nt <= 0 || !X || !tri) return CS_ERR_ARG;
  try {
    ClothTopo t;
    std::vector<int> bc(np, 0);
    build_topology(t, np, X, bc.data(), nt, tri, 0, nullptr, false);
    if (nnode) *nnode = t.nnode;
    if (!nodes) return CS_OK;
    if ((long long)cap < 3LL * t.nnode) return CS_ERR_CAPACITY;
    std::memcpy(nodes, t.node.data(), sizeof(int) * t.node.size());
    return CS_OK;
  } catch (...) {
    return CS_ERR_ARG;
  }
}

int cs_build_pattern(int np, int nq, const int* quad, int* row_ptr, int* col_idx, int cap, int* nb) {
  if (np <= 0 || nq < 0 || (nq > 0 && !quad)) return CS_ERR_ARG;
  try {
    ClothTopo t;
    build_pattern_only(t, np, nq, quad);
    if (nb) *nb = t.nb;
    if (row_ptr) std::memcpy(row_ptr, t.row_ptr.data(), sizeof(int) * t.row_ptr.size());
    if (!col_idx) return CS_OK;
    if (cap < t.nb) return CS_ERR_CAPACITY;
    std::memcpy(col_idx, t.col_idx.data(), sizeof(int) * t.col_idx.size());
    return CS_OK;
  } catch (...) {
    return CS_ERR_ARG;
  }
}

}  // extern "C"

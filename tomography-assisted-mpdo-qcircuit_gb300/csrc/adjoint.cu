// Reverse-mode gradient of an MPDO evolution (no counterpart in the
// reference, whose gate tensors detach the angles: SingleGates.py:181-185,
// YGates.py:66-68).  mpdo_program_grad evolves a circuit program, evaluates a
// loss L = Re Tr(rho H) for a Hermitian H given as a matrix-product operator,
// and returns dL/d(every gate / Kraus tensor of the program).
//
// Order of operations (the engine's own, which oracle/engine_path.py restates
// and pins against the reference order): a pending 2q gate is materialised by
// Householder QR of its left site (site := I_2 (x) Q', R' and the gate mix pushed
// into the right site) -- inside the QR sweep of a truncate() (Circuit.py:476-481,
// TNNOptimizer.py:87-108), or when another gate touches the pair; the SVD sweep
// (TNNOptimizer.py:111-134) decomposes the right site of each bond, its left
// neighbour being an isometry; the kappa pass (TNNOptimizer.py:164-197) keeps
// U S.  Every split keeps at most the numerical rank (singular values above
// rank_tol * s_0): the dropped directions change the state at the level of
// rank_tol^2, and without them every QR factor of the next sweep has full
// rank, where the QR adjoint is defined.  The 2q split's absolute cutoff is
// not applied (as in the engine's fused path).
//
// Memory: the chain is checkpointed at the start of every truncate segment;
// the reverse sweep re-runs one segment at a time with its intermediates
// recorded (QR factors, singular vectors, the two-site mixes) and
// back-propagates through it.
//
// Adjoints (cotangent Xbar = dL/dRe X + i dL/dIm X):
//   QR  A = QR:  Abar = [Qbar + Q copyltu(R Rbar^H - Qbar^H Q)] R^-H (wide A:
//                the trailing columns' R block adds Q (R_Y Rbar_Y^H) to Qbar)
//   split Y = U S V^H -> L = U_k S^1/2, R = S^-1/2 U_k^H Y: through the
//                eigen-decomposition of G = Y Y^H with the full basis U:
//                Gbar = U K U_k^H, K_ij = (U^H Ubar_k)_ij / (lam_j - lam_i)
//                (broadened), K_jj = lambar_j; Ybar = 2 herm(Gbar) Y + U_k S^-1/2 Rbar
//   kappa site := A V_k: Abar = Nbar V_k^H + A 2 herm(V C V_k^H),
//                C_ij = (V^H A^H Nbar)_ij / (lam_j - lam_i) for discarded i
//                (the kept block is a gauge of the Kraus leg and drops out).
#include "engine_core.cuh"

#include <stdexcept>

namespace mpdo {
namespace {

template <typename T> using CBuf = DBuf<cx<T>>;

template <typename T> CBuf<T> dcopy(Engine &e, const cx<T> *src, size_t n) {
  CBuf<T> b(e, n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(b.p, src, n * sizeof(cx<T>), cudaMemcpyDeviceToDevice, e.stream));
  return b;
}
// dst (M x N row-major) = conj(transpose of src (N x M row-major))
template <typename T> void adjoint_copy(Engine &e, cx<T> *dst, const cx<T> *src, int M, int N) {
  const int64_t d[4] = {1, 1, M, N};
  const int64_t st[4] = {0, 0, 1, M};
  copy4d<T>(e.stream, dst, src, d, st, 1);
}
template <typename T> std::vector<T> to_host(Engine &e, const T *p, size_t n) {
  std::vector<T> h(n);
  MPDO_CUDA_CHECK(cudaMemcpyAsync(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, e.stream));
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  return h;
}

enum RecKind { R_K1 = 1, R_PAIRQR, R_ABSORB, R_QR, R_SVD, R_KAPPA };

template <typename T> struct Rec {
  RecKind kind;
  int i = 0, op = -1, K = 1;
  int d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, d5 = 0;   // shapes, per kind
  int keep = 0;
  std::vector<double> t;                              // gate tensor (host)
  CBuf<T> A, B, C, D, E;
  DBuf<T> s;
};

template <typename T> struct Ctx {
  Engine &e;
  mpdo_chain_s *ch;
  const mpdo_program *prog;
  double rank_tol, beta;
  bool record = false;
  std::vector<Rec<T>> tape;
  std::vector<int> pend_op;                           // program op of each pending pair
  std::vector<DBuf<double2>> ggrad;                   // per program op
  Ctx(Engine &eng, mpdo_chain_s *c, const mpdo_program *p) : e(eng), ch(c), prog(p) {}
};

// replace site i by p; the old buffer is handed to `old` (when recording) or freed
template <typename T> void put_site(Ctx<T> &c, int i, cx<T> *p, int l, int a, int r, CBuf<T> *old) {
  Site &s = c.ch->s[i];
  if (old && c.record) {
    *old = CBuf<T>();
    old->e = &c.e;
    old->p = static_cast<cx<T> *>(s.p);
    old->n = s.elems();
  } else if (s.p) {
    dfree(c.e, s.p);
  }
  s.p = p;
  s.l = l; s.a = a; s.r = r;
}

template <typename T> const double *op_tensor(const Ctx<T> &c, int op) { return c.prog->kraus + c.prog->op_offset[op]; }

template <typename T> int rank_keep(Ctx<T> &c, const T *s_dev, int len, int cap) {
  std::vector<T> s = to_host<T>(c.e, s_dev, (size_t)len);
  int k = 0;
  const double thr = c.rank_tol * (len ? (double)s[0] : 0.0);
  while (k < len && (double)s[k] > thr) ++k;
  return std::max(1, std::min(k, cap));
}

// ------------------------------------------------------------ forward ----
template <typename T> void pairqr(Ctx<T> &c, int i);

template <typename T> void apply_1q(Ctx<T> &c, int site, int op) {
  Engine &e = c.e;
  if (site > 0 && c.ch->pend[site - 1].on) pairqr<T>(c, site - 1);
  if (site < c.ch->n - 1 && c.ch->pend[site].on) pairqr<T>(c, site);
  const int K = c.prog->op_k[op];
  const Site s = c.ch->s[site];
  CBuf<T> out(e, (size_t)s.l * 2 * s.a * K * s.r);
  kraus1q<T>(e.stream, static_cast<cx<T> *>(s.p), out.p, s.l, s.a, s.r, op_tensor(c, op), K);
  Rec<T> rec{R_K1};
  rec.i = site; rec.op = op; rec.K = K; rec.d0 = s.l; rec.d1 = s.a; rec.d2 = s.r;
  put_site<T>(c, site, out.release(), s.l, s.a * K, s.r, &rec.A);
  if (c.record) c.tape.push_back(std::move(rec));
}

template <typename T> void apply_2q(Ctx<T> &c, int i, int op) {
  for (int j = std::max(0, i - 1); j <= std::min(c.ch->n - 2, i + 1); ++j)
    if (c.ch->pend[j].on) pairqr<T>(c, j);
  Pend &p = c.ch->pend[i];
  const int K = c.prog->op_k[op];
  p.on = true;
  p.t.assign(op_tensor(c, op), op_tensor(c, op) + 32 * K);
  p.K = K;
  c.pend_op[i] = op;
  c.ch->bond[i] = 1;
}

// site i [b][s][a][m] -> At[(b,a)][(s,m)] = Q' R'; site i = I_2 (x) Q';
// W[s][k][t][c][r] = sum_m' R'[k][s m + m'] B[m'][t][c][r]; site i+1 = mix(W)
template <typename T> void pairqr(Ctx<T> &c, int i) {
  Engine &e = c.e;
  Pend pd = c.ch->pend[i];
  c.ch->pend[i].on = false;
  const int op = c.pend_op[i];
  const Site A = c.ch->s[i], Bs = c.ch->s[i + 1];
  const int b = A.l, a = A.a, m = A.r, cc = Bs.a, r = Bs.r, K = pd.K;
  const int mr = b * a, nc = 2 * m, kq = std::min(mr, nc);
  CBuf<T> At(e, (size_t)mr * nc);
  {
    const int64_t d[4] = {b, a, 2, m};
    const int64_t st[4] = {(int64_t)2 * a * m, m, (int64_t)a * m, 1};
    copy4d<T>(e.stream, At.p, static_cast<cx<T> *>(A.p), d, st, 0);
  }
  CBuf<T> Q(e, (size_t)mr * kq), R(e, (size_t)kq * nc);
  qr<T>(e, mr, nc, RM<T>(At.p, nc), Q.p, R.p);
  At.reset();
  CBuf<T> Si(e, (size_t)b * 2 * a * 2 * kq);
  blockdiag2<T>(e.stream, Si.p, Q.p, b, a, kq);
  const int ncol = 2 * cc * r;
  CBuf<T> W(e, (size_t)2 * kq * ncol);
  gemm<T>(e, kq, ncol, m, View<T>{R.p, (int64_t)m, 1, nc, 0, 1, 0}, RM<T>(static_cast<cx<T> *>(Bs.p), ncol), W.p,
          ncol, 2, (int64_t)kq * ncol);
  CBuf<T> Z(e, (size_t)2 * kq * 2 * cc * K * r);
  mix2q<T>(e.stream, W.p, Z.p, kq, cc, r, pd.t.data(), K);
  Rec<T> rec{R_PAIRQR};
  rec.i = i; rec.op = op; rec.K = K;
  rec.d0 = b; rec.d1 = a; rec.d2 = m; rec.d3 = cc; rec.d4 = r; rec.d5 = kq;
  put_site<T>(c, i, Si.release(), b, a, 2 * kq, &rec.A);
  put_site<T>(c, i + 1, Z.release(), 2 * kq, cc * K, r, &rec.B);
  if (c.record) {
    rec.C = std::move(Q);
    rec.D = std::move(R);
    rec.E = std::move(W);
    rec.t = pd.t;
    c.tape.push_back(std::move(rec));
  }
}

// site i := Rprev . site i
template <typename T> void absorb(Ctx<T> &c, int i, CBuf<T> &Rp, int rr, int rc) {
  Engine &e = c.e;
  const Site s = c.ch->s[i];
  if (s.l != rc) fail(MPDO_ERR_BAD_SHAPE, "adjoint: bond mismatch in absorb");
  const int ncol = 2 * s.a * s.r;
  CBuf<T> X(e, (size_t)rr * ncol);
  gemm<T>(e, rr, ncol, rc, RM<T>(Rp.p, rc), RM<T>(static_cast<cx<T> *>(s.p), ncol), X.p, ncol);
  Rec<T> rec{R_ABSORB};
  rec.i = i; rec.d0 = rr; rec.d1 = rc; rec.d2 = s.a; rec.d3 = s.r;
  put_site<T>(c, i, X.release(), rr, s.a, s.r, &rec.B);
  if (c.record) {
    rec.A = std::move(Rp);
    c.tape.push_back(std::move(rec));
  }
  Rp.reset();
}

// site i (rows x r) = Q R; site := Q; returns R
template <typename T> CBuf<T> qrstep(Ctx<T> &c, int i, int &kq_out) {
  Engine &e = c.e;
  const Site s = c.ch->s[i];
  const int mr = s.l * 2 * s.a, nc = s.r, kq = std::min(mr, nc);
  CBuf<T> Q(e, (size_t)mr * kq), R(e, (size_t)kq * nc);
  qr<T>(e, mr, nc, RM<T>(static_cast<cx<T> *>(s.p), nc), Q.p, R.p);
  Rec<T> rec{R_QR};
  rec.i = i; rec.d0 = mr; rec.d1 = nc; rec.d2 = kq;
  if (c.record) {
    rec.C = dcopy<T>(e, Q.p, (size_t)mr * kq);
    rec.D = dcopy<T>(e, R.p, (size_t)kq * nc);
  }
  put_site<T>(c, i, Q.release(), s.l, s.a, kq, nullptr);
  if (c.record) c.tape.push_back(std::move(rec));
  kq_out = kq;
  return R;
}

// bond idx-1|idx: Y = site idx (b x Nc) = U S V^H; L = U_k S^1/2 into site idx-1, R = S^-1/2 U_k^H Y
template <typename T> void svdstep(Ctx<T> &c, int idx, int chi) {
  Engine &e = c.e;
  const Site P = c.ch->s[idx - 1], S = c.ch->s[idx];
  const int b = S.l, Nc = 2 * S.a * S.r, rows_prev = P.l * 2 * P.a;
  const cx<T> *Y = static_cast<cx<T> *>(S.p);
  CBuf<T> U;
  DBuf<T> sg;
  right_svd<T>(e, Nc, b, CM<T>(Y, Nc, 1), U, sg);           // U: b x b column-major
  const int nsv = std::min(rows_prev, Nc);
  const int cap = chi > 0 ? std::min(chi, nsv) : nsv;
  const int k = rank_keep<T>(c, sg.p, std::min(b, Nc), cap);
  CBuf<T> L(e, (size_t)b * k), R(e, (size_t)k * Nc);
  {
    const int64_t d[4] = {1, 1, b, k};
    const int64_t st[4] = {0, 0, 1, b};
    copy4d<T>(e.stream, L.p, U.p, d, st, 0);
  }
  scale_matrix<T>(e.stream, L.p, b, k, k, sg.p, 0, 1);
  gemm<T>(e, k, Nc, b, RM<T>(U.p, b, 1), RM<T>(Y, Nc), R.p, Nc);
  scale_matrix<T>(e.stream, R.p, k, Nc, Nc, sg.p, 1, 2);
  CBuf<T> NP(e, (size_t)rows_prev * k);
  gemm<T>(e, rows_prev, k, b, RM<T>(static_cast<cx<T> *>(P.p), b), RM<T>(L.p, k), NP.p, k);
  Rec<T> rec{R_SVD};
  rec.i = idx; rec.keep = k; rec.d0 = rows_prev; rec.d1 = b; rec.d2 = Nc;
  put_site<T>(c, idx - 1, NP.release(), P.l, P.a, k, &rec.A);
  CBuf<T> Rsite = c.record ? dcopy<T>(e, R.p, (size_t)k * Nc) : CBuf<T>();
  put_site<T>(c, idx, R.release(), k, S.a, S.r, &rec.B);
  if (c.record) {
    rec.C = std::move(U);
    rec.s = std::move(sg);
    rec.D = std::move(L);
    rec.E = std::move(Rsite);
    c.tape.push_back(std::move(rec));
  }
}

// site i: A as (l, s, r) x a = U S V^H; site := A V_k
template <typename T> void kappastep(Ctx<T> &c, int i, int kappa) {
  Engine &e = c.e;
  const Site s = c.ch->s[i];
  if (s.a == 1 || (kappa > 0 && s.a <= kappa)) return;
  const int rows = s.l * 2 * s.r, a = s.a;
  CBuf<T> Am(e, (size_t)rows * a);
  {
    const int64_t d[4] = {s.l, 2, s.r, a};
    const int64_t st[4] = {(int64_t)2 * a * s.r, (int64_t)a * s.r, 1, s.r};
    copy4d<T>(e.stream, Am.p, static_cast<cx<T> *>(s.p), d, st, 0);
  }
  CBuf<T> V;
  DBuf<T> sg;
  right_svd<T>(e, rows, a, RM<T>(Am.p, a), V, sg);          // V: a x a column-major
  const int nsv = std::min(rows, a);
  const int k = rank_keep<T>(c, sg.p, nsv, kappa > 0 ? std::min(kappa, nsv) : nsv);
  CBuf<T> NM(e, (size_t)rows * k), NS(e, (size_t)rows * k);
  gemm<T>(e, rows, k, a, RM<T>(Am.p, a), CM<T>(V.p, a), NM.p, k);
  {
    const int64_t d[4] = {s.l, 2, k, s.r};
    const int64_t st[4] = {(int64_t)2 * s.r * k, (int64_t)s.r * k, 1, k};
    copy4d<T>(e.stream, NS.p, NM.p, d, st, 0);
  }
  Rec<T> rec{R_KAPPA};
  rec.i = i; rec.keep = k; rec.d0 = s.l; rec.d1 = s.r; rec.d2 = a;
  put_site<T>(c, i, NS.release(), s.l, k, s.r, nullptr);
  if (c.record) {
    rec.A = std::move(Am);
    rec.C = std::move(V);
    rec.s = std::move(sg);
    c.tape.push_back(std::move(rec));
  }
}

template <typename T> void materialize_pending(Ctx<T> &c) {
  for (int i = 0; i + 1 < c.ch->n; ++i)
    if (c.ch->pend[i].on) pairqr<T>(c, i);
}

template <typename T> void truncate(Ctx<T> &c, int chi, int kappa, bool noisy) {
  mpdo_chain_s *ch = c.ch;
  const int n = ch->n;
  if (chi > 0) {
    CBuf<T> Rp;
    int rr = 0, rc = 0;
    for (int i = 0; i < n - 1; ++i) {
      if (Rp.p) absorb<T>(c, i, Rp, rr, rc);
      if (ch->pend[i].on) {
        pairqr<T>(c, i);
        continue;
      }
      int kq = 0;
      rc = ch->s[i].r;
      Rp = qrstep<T>(c, i, kq);
      rr = kq;
    }
    if (Rp.p) absorb<T>(c, n - 1, Rp, rr, rc);
    for (int idx = n - 1; idx >= 1; --idx) svdstep<T>(c, idx, chi);
  }
  if (noisy) {
    materialize_pending<T>(c);
    for (int i = 0; i < n; ++i) kappastep<T>(c, i, kappa);
  }
}

template <typename T> void run_ops(Ctx<T> &c, int from, int to, bool last) {
  const mpdo_program &p = *c.prog;
  for (int j = from; j < to; ++j) {
    switch (p.op_kind[j]) {
      case MPDO_OP_1Q: apply_1q<T>(c, p.op_site[j], j); break;
      case MPDO_OP_2Q: apply_2q<T>(c, p.op_site[j], j); break;
      case MPDO_OP_TRUNCATE: truncate<T>(c, p.chi, p.kappa, p.noisy != 0); break;
      case MPDO_OP_KAPPA:
        materialize_pending<T>(c);
        for (int i = 0; i < c.ch->n; ++i) kappastep<T>(c, i, p.kappa);
        break;
      default: fail(MPDO_ERR_INVALID, "unknown op kind");
    }
  }
  if (last) materialize_pending<T>(c);
}

// ------------------------------------------------------------ adjoints --
// Abar of A = QR (mr x nc) given Qbar (mr x kq) and Rbar (kq x nc, may be null)
template <typename T>
CBuf<T> qr_bwd(Engine &e, int mr, int nc, const cx<T> *Q, const cx<T> *R, const cx<T> *Qb, const cx<T> *Rb) {
  const int kq = std::min(mr, nc);
  const cx<T> one = cmk<T>(T(1), T(0)), mone = cmk<T>(T(-1), T(0));
  CBuf<T> Ab(e, (size_t)mr * nc);
  if (mr < nc) fill_zero<T>(e.stream, Ab.p, (size_t)mr * nc);
  CBuf<T> Qb2 = dcopy<T>(e, Qb, (size_t)mr * kq);
  if (mr < nc && Rb) {
    // trailing block Y = Q R_Y: Ybar = Q Rbar_Y; Qbar += Q (R_Y Rbar_Y^H)
    const int ny = nc - mr;
    gemm<T>(e, mr, ny, kq, RM<T>(Q, kq), View<T>{Rb + mr, 0, 1, nc, 0, 1, 0}, Ab.p + mr, nc);
    CBuf<T> tmp(e, (size_t)kq * kq);
    gemm<T>(e, kq, kq, ny, View<T>{R + mr, 0, 1, nc, 0, 1, 0}, View<T>{Rb + mr, 0, 1, 1, 0, nc, 1}, tmp.p, kq);
    gemm<T>(e, mr, kq, kq, RM<T>(Q, kq), RM<T>(tmp.p, kq), Qb2.p, kq, 1, 0, one);
  }
  // M = R_X Rbar_X^H - Qbar^H Q (kq x kq), R_X = first kq columns of R
  CBuf<T> M(e, (size_t)kq * kq);
  if (Rb)
    gemm<T>(e, kq, kq, kq, RM<T>(R, nc), View<T>{Rb, 0, 1, 1, 0, nc, 1}, M.p, kq);
  else
    fill_zero<T>(e.stream, M.p, (size_t)kq * kq);
  gemm<T>(e, kq, kq, mr, CM<T>(Qb2.p, kq, 1), RM<T>(Q, kq), M.p, kq, 1, 0, one, mone);
  copyltu<T>(e.stream, M.p, kq);
  gemm<T>(e, mr, kq, kq, RM<T>(Q, kq), RM<T>(M.p, kq), Qb2.p, kq, 1, 0, one);
  trsm_rh<T>(e.stream, Qb2.p, mr, kq, kq, R, nc);
  MPDO_CUDA_CHECK(cudaMemcpy2DAsync(Ab.p, nc * sizeof(cx<T>), Qb2.p, kq * sizeof(cx<T>), kq * sizeof(cx<T>), mr,
                                    cudaMemcpyDeviceToDevice, e.stream));
  return Ab;
}

template <typename T> struct Cot {
  std::vector<CBuf<T>> site;   // cotangent of each current site tensor
  CBuf<T> Rbar;                // cotangent of the R carried by the QR sweep
};

template <typename T> void back_k1(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  const int L = r.d0, Aa = r.d1, R = r.d2;
  CBuf<T> Ab(e, (size_t)L * 2 * Aa * R);
  const cx<T> *Ob = g.site[r.i].p;
  kraus1q_bwd<T>(e.stream, Ob, Ab.p, L, Aa, R, op_tensor(c, r.op), r.K);
  kraus1q_grad<T>(e.stream, Ob, r.A.p, L, Aa, R, r.K, c.ggrad[r.op].p);
  g.site[r.i] = std::move(Ab);
}

template <typename T> void back_pairqr(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  const int b = r.d0, a = r.d1, m = r.d2, cc = r.d3, rr = r.d4, kq = r.d5, K = r.K;
  const int mr = b * a, nc = 2 * m, ncol = 2 * cc * rr;
  const cx<T> one = cmk<T>(T(1), T(0));
  CBuf<T> &Sb = g.site[r.i], &Zb = g.site[r.i + 1];
  // mix: Wbar and the gate tensor's gradient
  CBuf<T> Wb(e, (size_t)2 * kq * ncol);
  mix2q_bwd<T>(e.stream, Zb.p, Wb.p, kq, cc, rr, r.t.data(), K);
  mix2q_grad<T>(e.stream, Zb.p, r.E.p, kq, cc, rr, K, c.ggrad[r.op].p);
  // Rbar'[k][s m + m'] = sum_col Wbar_s[k][col] conj(B[m'][col]); Bbar = sum_s R'_s^H Wbar_s
  CBuf<T> Rb(e, (size_t)kq * nc), Bb(e, (size_t)m * ncol);
  gemm<T>(e, kq, m, ncol, View<T>{Wb.p, (int64_t)kq * ncol, 1, ncol, 0, 1, 0}, CM<T>(r.B.p, ncol, 1), Rb.p, nc, 2,
          (int64_t)m);
  for (int s = 0; s < 2; ++s)
    gemm<T>(e, m, ncol, kq, View<T>{r.D.p + (size_t)s * m, 0, 1, 1, 0, nc, 1},
            RM<T>(Wb.p + (size_t)s * kq * ncol, ncol), Bb.p, ncol, 1, 0, s ? one : czero<T>());
  // blockdiag: Qbar'
  CBuf<T> Qb(e, (size_t)mr * kq);
  blockdiag2_bwd<T>(e.stream, Sb.p, Qb.p, b, a, kq);
  CBuf<T> Atb = qr_bwd<T>(e, mr, nc, r.C.p, r.D.p, Qb.p, Rb.p);
  CBuf<T> Ab(e, (size_t)b * 2 * a * m);
  {  // At[(b,a)][(s,m)] -> A[b][s][a][m]
    const int64_t d[4] = {b, 2, a, m};
    const int64_t st[4] = {(int64_t)a * nc, m, nc, 1};
    copy4d<T>(e.stream, Ab.p, Atb.p, d, st, 0);
  }
  g.site[r.i] = std::move(Ab);
  g.site[r.i + 1] = std::move(Bb);
}

template <typename T> void back_absorb(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  const int rr = r.d0, rc = r.d1, ncol = 2 * r.d2 * r.d3;
  CBuf<T> &Xb = g.site[r.i];
  CBuf<T> Ab(e, (size_t)rc * ncol), Rb(e, (size_t)rr * rc);
  gemm<T>(e, rc, ncol, rr, CM<T>(r.A.p, rc, 1), RM<T>(Xb.p, ncol), Ab.p, ncol);       // Rprev^H Xbar
  gemm<T>(e, rr, rc, ncol, RM<T>(Xb.p, ncol), CM<T>(r.B.p, ncol, 1), Rb.p, rc);        // Xbar A^H
  g.site[r.i] = std::move(Ab);
  g.Rbar = std::move(Rb);
}

template <typename T> void back_qr(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  CBuf<T> Ab = qr_bwd<T>(e, r.d0, r.d1, r.C.p, r.D.p, g.site[r.i].p, g.Rbar.p);
  g.Rbar.reset();
  g.site[r.i] = std::move(Ab);
}

template <typename T> void back_svd(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  const int rows_prev = r.d0, b = r.d1, Nc = r.d2, k = r.keep;
  const cx<T> one = cmk<T>(T(1), T(0));
  CBuf<T> &Pb1 = g.site[r.i - 1], &Rbar = g.site[r.i];
  const cx<T> *P = r.A.p, *Y = r.B.p, *U = r.C.p, *L = r.D.p, *R = r.E.p;
  const T *s = r.s.p;
  CBuf<T> Pb(e, (size_t)rows_prev * b), Lb(e, (size_t)b * k);
  gemm<T>(e, rows_prev, b, k, RM<T>(Pb1.p, k), CM<T>(L, k, 1), Pb.p, b);                // Pbar' L^H
  gemm<T>(e, b, k, rows_prev, CM<T>(P, b, 1), RM<T>(Pb1.p, k), Lb.p, k);                // P^H Pbar'
  DBuf<double> dd(e, 2 * (size_t)k);
  redot<T>(e.stream, Lb.p, L, k, b, k, 1, dd.p);
  redot<T>(e.stream, Rbar.p, R, k, Nc, 1, Nc, dd.p + k);
  // Ubar_k = Lbar S^1/2 + Y Rbar^H S^-1/2
  CBuf<T> Ub = dcopy<T>(e, Lb.p, (size_t)b * k), T2(e, (size_t)b * k);
  scale_matrix<T>(e.stream, Ub.p, b, k, k, s, 0, 1);
  gemm<T>(e, b, k, Nc, RM<T>(Y, Nc), CM<T>(Rbar.p, Nc, 1), T2.p, k);
  scale_matrix<T>(e.stream, T2.p, b, k, k, s, 0, 2);
  axpy<T>(e.stream, Ub.p, T2.p, (int64_t)b * k, 1.0);
  // K = F o (U^H Ubar_k) + diag(lambar); Gbar = (U K) U_k^H
  CBuf<T> UhUb(e, (size_t)b * k), Km(e, (size_t)b * k), UK(e, (size_t)b * k), Gb(e, (size_t)b * b),
      H2(e, (size_t)b * b);
  gemm<T>(e, b, k, b, RM<T>(U, b, 1), RM<T>(Ub.p, k), UhUb.p, k);
  split_K<T>(e.stream, UhUb.p, s, b, k, dd.p, dd.p + k, c.beta, Km.p);
  gemm<T>(e, b, k, b, CM<T>(U, b), RM<T>(Km.p, k), UK.p, k);
  gemm<T>(e, b, b, k, RM<T>(UK.p, k), RM<T>(U, b, 1), Gb.p, b);
  adjoint_copy<T>(e, H2.p, Gb.p, b, b);
  axpy<T>(e.stream, H2.p, Gb.p, (int64_t)b * b, 1.0);
  // Ybar = H2 Y + U_k S^-1/2 Rbar
  CBuf<T> Yb(e, (size_t)b * Nc), Us(e, (size_t)b * k);
  gemm<T>(e, b, Nc, b, RM<T>(H2.p, b), RM<T>(Y, Nc), Yb.p, Nc);
  {
    const int64_t d[4] = {1, 1, b, k};
    const int64_t st[4] = {0, 0, 1, b};
    copy4d<T>(e.stream, Us.p, U, d, st, 0);
  }
  scale_matrix<T>(e.stream, Us.p, b, k, k, s, 0, 2);
  gemm<T>(e, b, Nc, k, RM<T>(Us.p, k), RM<T>(Rbar.p, Nc), Yb.p, Nc, 1, 0, one);
  g.site[r.i - 1] = std::move(Pb);
  g.site[r.i] = std::move(Yb);
}

template <typename T> void back_kappa(Ctx<T> &c, Cot<T> &g, Rec<T> &r) {
  Engine &e = c.e;
  const int l = r.d0, rr = r.d1, a = r.d2, k = r.keep, rows = l * 2 * rr;
  const cx<T> one = cmk<T>(T(1), T(0));
  const cx<T> *Am = r.A.p, *V = r.C.p;
  // Nbar [l][s][k][r] -> (l, s, r) x k
  CBuf<T> Nb(e, (size_t)rows * k);
  {
    const int64_t d[4] = {l, 2, rr, k};
    const int64_t st[4] = {(int64_t)2 * k * rr, (int64_t)k * rr, 1, rr};
    copy4d<T>(e.stream, Nb.p, g.site[r.i].p, d, st, 0);
  }
  CBuf<T> X(e, (size_t)a * k), VhX(e, (size_t)a * k), C(e, (size_t)a * k), VC(e, (size_t)a * k),
      Hb(e, (size_t)a * a), H2(e, (size_t)a * a), Ab(e, (size_t)rows * a);
  gemm<T>(e, a, k, rows, CM<T>(Am, a, 1), RM<T>(Nb.p, k), X.p, k);                      // A^H Nbar
  gemm<T>(e, a, k, a, RM<T>(V, a, 1), RM<T>(X.p, k), VhX.p, k);                         // V^H X
  kappa_C<T>(e.stream, VhX.p, r.s.p, a, k, c.beta, C.p);
  gemm<T>(e, a, k, a, CM<T>(V, a), RM<T>(C.p, k), VC.p, k);
  gemm<T>(e, a, a, k, RM<T>(VC.p, k), RM<T>(V, a, 1), Hb.p, a);                         // V C V_k^H
  adjoint_copy<T>(e, H2.p, Hb.p, a, a);
  axpy<T>(e.stream, H2.p, Hb.p, (int64_t)a * a, 1.0);
  gemm<T>(e, rows, a, k, RM<T>(Nb.p, k), RM<T>(V, a, 1), Ab.p, a);                      // Nbar V_k^H
  gemm<T>(e, rows, a, a, RM<T>(Am, a), RM<T>(H2.p, a), Ab.p, a, 1, 0, one);             // + A H2
  CBuf<T> As(e, (size_t)rows * a);
  {  // (l, s, r) x a -> [l][s][a][r]
    const int64_t d[4] = {l, 2, a, rr};
    const int64_t st[4] = {(int64_t)2 * rr * a, (int64_t)rr * a, 1, a};
    copy4d<T>(e.stream, As.p, Ab.p, d, st, 0);
  }
  g.site[r.i] = std::move(As);
}

template <typename T> void backprop(Ctx<T> &c, Cot<T> &g) {
  for (int j = (int)c.tape.size() - 1; j >= 0; --j) {
    Rec<T> &r = c.tape[j];
    switch (r.kind) {
      case R_K1: back_k1<T>(c, g, r); break;
      case R_PAIRQR: back_pairqr<T>(c, g, r); break;
      case R_ABSORB: back_absorb<T>(c, g, r); break;
      case R_QR: back_qr<T>(c, g, r); break;
      case R_SVD: back_svd<T>(c, g, r); break;
      case R_KAPPA: back_kappa<T>(c, g, r); break;
    }
    c.tape.pop_back();
  }
}

// ------------------------------------------------ MPO readout and adjoint --
// Loss Re Tr(rho H), H = MPO with site tensors W_k[Dl][Dr][s'][s]; site
// cotangents Abar_k = 2 sum_D' G_k[D'] Fr_{k+1}[D'] (H Hermitian).
template <typename T>
double mpo_loss_grad(Ctx<T> &c, const int *Dd, const cx<T> *Wdev, const std::vector<size_t> &woff, Cot<T> &g) {
  Engine &e = c.e;
  mpdo_chain_s *ch = c.ch;
  const int n = ch->n;
  const cx<T> one = cmk<T>(T(1), T(0)), two = cmk<T>(T(2), T(0));
  std::vector<CBuf<T>> E(n + 1), Fr(n + 1);
  E[0] = CBuf<T>(e, 1);
  Fr[n] = CBuf<T>(e, 1);
  {
    const cx<T> h = one;
    MPDO_CUDA_CHECK(cudaMemcpyAsync(E[0].p, &h, sizeof(h), cudaMemcpyHostToDevice, e.stream));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(Fr[n].p, &h, sizeof(h), cudaMemcpyHostToDevice, e.stream));
    MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  }
  // left: G[D'][l'][s'][a][r] = sum_{D,s} W[D][D'][s'][s] sum_l E[D][l][l'] A[l][s][a][r]
  auto left_G = [&](int k, CBuf<T> &G) {
    const Site s = ch->s[k];
    const int D = Dd[k], D2 = Dd[k + 1], l = s.l, ar = s.a * s.r;
    const cx<T> *A = static_cast<cx<T> *>(s.p);
    CBuf<T> F(e, (size_t)D * l * 2 * ar);
    gemm<T>(e, l, 2 * ar, l, CM<T>(E[k].p, l, 0, (int64_t)l * l), RM<T>(A, 2 * ar), F.p, 2 * ar, D,
            (int64_t)l * 2 * ar);
    G = CBuf<T>(e, (size_t)D2 * l * 2 * ar);
    mpo_mix<T>(e.stream, F.p, G.p, Wdev + woff[k], D, D2, (int64_t)D2 * 4, 4, l, ar);
  };
  for (int k = 0; k < n; ++k) {
    const Site s = ch->s[k];
    const int D2 = Dd[k + 1], l = s.l, R = s.r;
    CBuf<T> G;
    left_G(k, G);
    E[k + 1] = CBuf<T>(e, (size_t)D2 * R * R);
    gemm<T>(e, R, R, l * 2 * s.a, CM<T>(G.p, R, 0, (int64_t)l * 2 * s.a * R),
            RM<T>(static_cast<cx<T> *>(s.p), R, 1), E[k + 1].p, R, D2, (int64_t)R * R);
  }
  const double loss = (double)to_host<cx<T>>(e, E[n].p, 1)[0].x;
  // right: Fr[D][l][l'] = sum J[D][l][(s' a r')] conj(A[l'][(s' a r')]),
  // J = sum_{D',s} W[D][D'][s'][s] (A . Fr'[D'])
  for (int k = n - 1; k >= 1; --k) {
    const Site s = ch->s[k];
    const int D = Dd[k], D2 = Dd[k + 1], l = s.l, R = s.r, ar = s.a * s.r;
    const cx<T> *A = static_cast<cx<T> *>(s.p);
    CBuf<T> H(e, (size_t)D2 * l * 2 * ar), J(e, (size_t)D * l * 2 * ar);
    gemm<T>(e, l * 2 * s.a, R, R, RM<T>(A, R), RM<T>(Fr[k + 1].p, R, 0, (int64_t)R * R), H.p, R, D2,
            (int64_t)l * 2 * ar);
    mpo_mix<T>(e.stream, H.p, J.p, Wdev + woff[k], D2, D, 4, (int64_t)D2 * 4, l, ar);
    Fr[k] = CBuf<T>(e, (size_t)D * l * l);
    gemm<T>(e, l, l, 2 * ar, RM<T>(J.p, 2 * ar, 0, (int64_t)l * 2 * ar), CM<T>(A, 2 * ar, 1), Fr[k].p, l, D,
            (int64_t)l * l);
  }
  g.site.clear();
  g.site.resize(n);
  for (int k = 0; k < n; ++k) {
    const Site s = ch->s[k];
    const int D2 = Dd[k + 1], l = s.l, R = s.r;
    CBuf<T> G;
    left_G(k, G);
    CBuf<T> Ab(e, s.elems());
    for (int d = 0; d < D2; ++d)
      gemm<T>(e, l * 2 * s.a, R, R, RM<T>(G.p + (size_t)d * l * 2 * s.a * R, R),
              RM<T>(Fr[k + 1].p + (size_t)d * R * R, R), Ab.p, R, 1, 0, d ? one : czero<T>(), two);
    g.site[k] = std::move(Ab);
  }
  return loss;
}

template <typename T> void clone_into(Engine &e, mpdo_chain_s *dst, const mpdo_chain_s *src) {
  for (auto &s : dst->s)
    if (s.p) dfree(e, s.p);
  *dst = *src;
  for (int i = 0; i < dst->n; ++i) {
    const size_t bytes = src->s[i].elems() * sizeof(cx<T>);
    void *p = dalloc(e, bytes);
    MPDO_CUDA_CHECK(cudaMemcpyAsync(p, src->s[i].p, bytes, cudaMemcpyDeviceToDevice, e.stream));
    dst->s[i].p = p;
  }
}

template <typename T> void free_chain(Engine &e, mpdo_chain_s *ch) {
  for (auto &s : ch->s)
    if (s.p) { dfree(e, s.p); s.p = nullptr; }
}

template <typename T>
void program_grad(mpdo_engine_s *eng, const mpdo_program *prog, const int *Dd, const double *mpo, double rank_tol,
                  double beta, double *loss_out, double *grad_out, double *phase_ms) {
  Engine &e = eng->e;
  const int n = prog->n;
  if (!prog->connected) fail(MPDO_ERR_INVALID, "the adjoint needs a connected chain (connected = 1)");
  if (prog->max_err >= 0) fail(MPDO_ERR_INVALID, "the adjoint supports chi / kappa caps only (max_err < 0)");
  for (int k = 0; k <= n; ++k)
    if (Dd[k] < 1 || Dd[k] > 64) fail(MPDO_ERR_INVALID, "MPO bond dimensions must be in [1, 64]");
  if (Dd[0] != 1 || Dd[n] != 1) fail(MPDO_ERR_INVALID, "the MPO's outer bonds must have dimension 1");
  // chain
  mpdo_chain_s chain;
  chain.eng = eng;
  chain.n = n;
  chain.dtype = prog->dtype;
  chain.s.assign(n, Site{});
  chain.bond.assign(std::max(0, n - 1), 1);
  chain.pend.assign(std::max(0, n - 1), Pend{});
  chain.pend1.assign(n, Pend{});
  for (int i = 0; i < n; ++i) {
    cx<T> h[2] = {cmk<T>((T)prog->vectors[4 * i], (T)prog->vectors[4 * i + 1]),
                  cmk<T>((T)prog->vectors[4 * i + 2], (T)prog->vectors[4 * i + 3])};
    cx<T> *p = static_cast<cx<T> *>(dalloc(e, sizeof(h)));
    MPDO_CUDA_CHECK(cudaMemcpyAsync(p, h, sizeof(h), cudaMemcpyHostToDevice, e.stream));
    chain.s[i] = Site{p, 1, 1, 1};
  }
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  Ctx<T> c(e, &chain, prog);
  c.rank_tol = rank_tol;
  c.beta = beta;
  c.pend_op.assign(std::max(0, n - 1), -1);
  c.ggrad.resize(prog->nops);
  for (int j = 0; j < prog->nops; ++j) {
    const int kind = prog->op_kind[j];
    if (kind == MPDO_OP_1Q || kind == MPDO_OP_2Q) {
      const size_t cnt = (size_t)(kind == MPDO_OP_1Q ? 4 : 16) * prog->op_k[j];
      c.ggrad[j] = DBuf<double2>(e, cnt);
      MPDO_CUDA_CHECK(cudaMemsetAsync(c.ggrad[j].p, 0, cnt * sizeof(double2), e.stream));
    }
  }
  // MPO on the device
  std::vector<size_t> woff(n + 1, 0);
  for (int k = 0; k < n; ++k) woff[k + 1] = woff[k] + (size_t)Dd[k] * Dd[k + 1] * 4;
  std::vector<cx<T>> wh(woff[n]);
  for (size_t q = 0; q < wh.size(); ++q) wh[q] = cmk<T>((T)mpo[2 * q], (T)mpo[2 * q + 1]);
  CBuf<T> Wd(e, std::max<size_t>(1, wh.size()));
  MPDO_CUDA_CHECK(cudaMemcpyAsync(Wd.p, wh.data(), wh.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, e.stream));
  // segments end at truncate / kappa ops
  std::vector<int> seg_end;
  for (int j = 0; j < prog->nops; ++j)
    if (prog->op_kind[j] == MPDO_OP_TRUNCATE || prog->op_kind[j] == MPDO_OP_KAPPA) seg_end.push_back(j + 1);
  if (seg_end.empty() || seg_end.back() != prog->nops) seg_end.push_back(prog->nops);
  const int nseg = (int)seg_end.size();
  std::vector<mpdo_chain_s> ckpt(nseg);
  std::vector<std::vector<int>> ck_pend(nseg);
  // phase events: forward (with checkpoints), readout and its adjoint, reverse sweep
  cudaEvent_t ev[4];
  for (auto &x : ev) MPDO_CUDA_CHECK(cudaEventCreate(&x));
  MPDO_CUDA_CHECK(cudaEventRecord(ev[0], e.stream));
  // forward with checkpoints
  c.record = false;
  for (int sgi = 0; sgi < nseg; ++sgi) {
    ckpt[sgi].s.clear();
    clone_into<T>(e, &ckpt[sgi], &chain);
    ck_pend[sgi] = c.pend_op;
    run_ops<T>(c, sgi ? seg_end[sgi - 1] : 0, seg_end[sgi], sgi == nseg - 1);
  }
  MPDO_CUDA_CHECK(cudaEventRecord(ev[1], e.stream));
  Cot<T> g;
  *loss_out = mpo_loss_grad<T>(c, Dd, Wd.p, woff, g);
  MPDO_CUDA_CHECK(cudaEventRecord(ev[2], e.stream));
  // reverse sweep, one segment at a time
  for (int sgi = nseg - 1; sgi >= 0; --sgi) {
    clone_into<T>(e, &chain, &ckpt[sgi]);
    free_chain<T>(e, &ckpt[sgi]);
    c.pend_op = ck_pend[sgi];
    c.record = true;
    c.tape.clear();
    run_ops<T>(c, sgi ? seg_end[sgi - 1] : 0, seg_end[sgi], sgi == nseg - 1);
    c.record = false;
    for (int i = 0; i < n; ++i)
      if (g.site[i].n != chain.s[i].elems()) fail(MPDO_ERR_BAD_SHAPE, "adjoint: recomputed segment changed shape");
    backprop<T>(c, g);
  }
  free_chain<T>(e, &chain);
  MPDO_CUDA_CHECK(cudaEventRecord(ev[3], e.stream));
  check_status(e);
  MPDO_CUDA_CHECK(cudaStreamSynchronize(e.stream));
  if (phase_ms)
    for (int q = 0; q < 3; ++q) {
      float ms = 0;
      MPDO_CUDA_CHECK(cudaEventElapsedTime(&ms, ev[q], ev[q + 1]));
      phase_ms[q] = ms;
    }
  for (auto &x : ev) cudaEventDestroy(x);
  if (e.first_status) {
    const int fs = e.first_status;
    e.first_status = 0;
    fail(fs == DEV_NONFINITE ? MPDO_ERR_NONFINITE : MPDO_ERR_NOT_CONVERGED,
         fs == DEV_NONFINITE ? "non-finite value met in a factorisation" : "Jacobi sweep limit reached");
  }
  // gate gradients to host
  for (int j = 0; j < prog->nops; ++j) {
    if (!c.ggrad[j].p) continue;
    std::vector<double2> h = to_host<double2>(e, c.ggrad[j].p, c.ggrad[j].n);
    double *dst = grad_out + prog->op_offset[j];
    for (size_t q = 0; q < h.size(); ++q) { dst[2 * q] = h[q].x; dst[2 * q + 1] = h[q].y; }
  }
}

}  // namespace
}  // namespace mpdo

using namespace mpdo;

extern "C" mpdo_status mpdo_program_grad(mpdo_engine_t eng, const mpdo_program *prog, const int *mpo_dims,
                                         const double *mpo, double rank_tol, double broadening, double *loss_out,
                                         double *grad_out, double *phase_ms) {
  return guard([&] {
    if (!eng || !prog || !mpo_dims || !mpo || !loss_out || !grad_out) fail(MPDO_ERR_INVALID, "NULL argument");
    if (prog->n < 2) fail(MPDO_ERR_INVALID, "n must be >= 2");
    if (!(rank_tol > 0 && rank_tol < 1)) fail(MPDO_ERR_INVALID, "rank_tol must be in (0, 1)");
    if (!(broadening >= 0)) fail(MPDO_ERR_INVALID, "broadening must be >= 0");
    MPDO_CUDA_CHECK(cudaSetDevice(eng->e.device));
    if (prog->dtype == MPDO_C64)
      program_grad<float>(eng, prog, mpo_dims, mpo, rank_tol, broadening, loss_out, grad_out, phase_ms);
    else
      program_grad<double>(eng, prog, mpo_dims, mpo, rank_tol, broadening, loss_out, grad_out, phase_ms);
  });
}

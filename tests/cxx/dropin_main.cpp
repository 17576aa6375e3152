// A DelFEM2-style caller written against delfem2::gb300 (include/dfm2g.hpp):
// the sequence of examples_oldgl_glfw/618_Fem3Tet/main.cpp:234-319 —
// pattern, Initialize/SetPattern, SetPattern0, setZero, element matrices on the
// host + Merge, SetFixedBC, CopyValue, Decompose, Solve_PCG — on an n^3 voxel
// block. Prints "iterations <k> residual <rel> xsum <sum(x)>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dfm2g.hpp"

namespace g = delfem2::gb300;

// K_e of a linear tet: vol (lambda dN_i[a] dN_j[b] + myu dN_j[a] dN_i[b] + myu dN_i.dN_j delta_ab)
static void emat_tet(const double P[4][3], double myu, double lam, double emat[4][4][3][3], double *vol_out) {
  const double *p0 = P[0];
  double a[3], b[3], c[3];
  for (int d = 0; d < 3; ++d) {
    a[d] = P[1][d] - p0[d];
    b[d] = P[2][d] - p0[d];
    c[d] = P[3][d] - p0[d];
  }
  const double vol = (a[0] * (b[1] * c[2] - c[1] * b[2]) - a[1] * (b[0] * c[2] - c[0] * b[2]) +
                      a[2] * (b[0] * c[1] - c[0] * b[1])) / 6.0;
  double dN[4][3];
  for (int k = 0; k < 4; ++k) {
    const double *u0 = P[(k + 1) % 4], *u1 = P[(k + 2) % 4], *u2 = P[(k + 3) % 4];
    const double ux = u1[0] - u0[0], uy = u1[1] - u0[1], uz = u1[2] - u0[2];
    const double wx = u2[0] - u0[0], wy = u2[1] - u0[1], wz = u2[2] - u0[2];
    const double s = ((k % 2) ? 1.0 : -1.0) / (6.0 * vol);
    dN[k][0] = s * (uy * wz - uz * wy);
    dN[k][1] = s * (uz * wx - ux * wz);
    dN[k][2] = s * (ux * wy - uy * wx);
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const double dd = dN[i][0] * dN[j][0] + dN[i][1] * dN[j][1] + dN[i][2] * dN[j][2];
      for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s)
          emat[i][j][r][s] = vol * (lam * dN[i][r] * dN[j][s] + myu * dN[j][r] * dN[i][s] + (r == s ? myu * dd : 0));
    }
  *vol_out = vol;
}

// A generic PCG written against the ADL primitives only, step for step as the
// reference's Solve_PCG<MAT, VEC, PREC> (lsitrsol.h:80-148): x = 0; history of
// |r| starting with |r0|; early return when |r0|^2 < 1e-30; Ap shares Pr's
// storage; stop when |r|/|r0| < tol; one more |r| entry when max_it runs out.
// It exercises the compatibility path of dfm2g.hpp with device vectors (every
// Dot is a device reduction read back to the host). Returns the history.
template <class MAT, class VEC, class PREC>
static std::vector<double> generic_pcg(VEC &r, VEC &x, VEC &Pr, VEC &p, double tol, unsigned max_it, const MAT &K,
                                       const PREC &M) {
  std::vector<double> hist;
  x.setZero();
  const double rr0 = Dot(r, r);
  hist.push_back(std::sqrt(rr0));
  if (rr0 < 1.0e-30) return hist;
  const double inv_rr0 = 1.0 / rr0;
  Pr = r;
  SolvePrecond(Pr, M);
  p = Pr;
  double rz = Dot(r, Pr);
  for (unsigned it = 0; it < max_it; ++it) {
    VEC &Ap = Pr;
    AddMatVec(Ap, 0.0, 1.0, K, p);
    const double alpha = rz / Dot(p, Ap);
    AddScaledVec(r, -alpha, Ap);
    AddScaledVec(x, alpha, p);
    const double rr = Dot(r, r);
    hist.push_back(std::sqrt(rr));
    if (std::sqrt(rr * inv_rr0) < tol) return hist;
    Pr = r;
    SolvePrecond(Pr, M);
    const double rz1 = Dot(r, Pr);
    ScaleAndAddVec(p, rz1 / rz, Pr);
    rz = rz1;
  }
  hist.push_back(std::sqrt(Dot(r, r)));
  return hist;
}

int main(int argc, char **argv) {
  const unsigned n = argc > 1 ? (unsigned)atoi(argv[1]) : 8;
  const size_t np = (size_t)(n + 1) * (n + 1) * (n + 1), ntet = (size_t)n * n * n * 6;
  std::vector<double> xyz(np * 3);
  std::vector<unsigned> tet(ntet * 4);
  g::check(dfm2g_mesh_tet_voxel_grid(n, n, n, 1.0 / n, xyz.data(), tet.data()), "mesh");
  std::vector<unsigned> psup_ind(np + 1);
  size_t npsup = 0;
  g::check(dfm2g_psup_count(tet.data(), ntet, 4, np, psup_ind.data(), &npsup), "psup");
  std::vector<unsigned> psup(npsup);
  g::check(dfm2g_psup_fill(tet.data(), ntet, 4, np, psup_ind.data(), psup.data()), "psup");

  g::CMatrixSparse<double> K;
  K.Initialize(np, 3, true);
  K.SetPattern(psup_ind.data(), psup_ind.size(), psup.data(), psup.size());
  g::CPreconditionerILU<double> ilu;
  ilu.SetPattern0(K);
  K.setZero();

  const double E = 1.0, nu = 0.3, rho = 1.0, gz = -1e-3;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu)), myu = E / (2 * (1 + nu));
  std::vector<double> b(np * 3, 0.0), emats(ntet * 144);
  for (size_t e = 0; e < ntet; ++e) {
    double P[4][3], vol;
    for (int k = 0; k < 4; ++k)
      for (int d = 0; d < 3; ++d) P[k][d] = xyz[tet[e * 4 + k] * 3 + d];
    emat_tet(P, myu, lam, reinterpret_cast<double(*)[4][3][3]>(&emats[e * 144]), &vol);
    for (int k = 0; k < 4; ++k) b[tet[e * 4 + k] * 3 + 2] += vol * rho * gz * 0.25;
  }
  // one element through the single-element Merge (the reference's call shape),
  // the rest batched
  std::vector<unsigned> buf;
  if (!g::Merge<4, 4, 3, 3, double>(K, &tet[0], &tet[0],
                                    reinterpret_cast<const double(*)[4][3][3]>(&emats[0]), buf))
    return 2;
  K.MergeBatch((unsigned)ntet - 1, 4, tet.data() + 4, emats.data() + 144);

  std::vector<int> bc(np * 3, 0);
  for (size_t p = 0; p < np; ++p)
    if (xyz[p * 3 + 2] == 0.0) bc[p * 3] = bc[p * 3 + 1] = bc[p * 3 + 2] = 1;
  K.SetFixedBC(bc.data());
  for (size_t i = 0; i < b.size(); ++i)
    if (bc[i]) b[i] = 0.0;
  ilu.CopyValue(K);
  if (!ilu.Decompose()) return 3;

  std::vector<double> r = b, x(b.size()), Pr(b.size()), p(b.size());
  const std::vector<double> hist = g::Solve_PCG(g::VectorView(r), g::VectorView(x), g::VectorView(Pr),
                                                g::VectorView(p), 1e-10, 1000, K, ilu);
  // true residual |b - K x| / |b|
  std::vector<double> Kx(b.size(), 0.0);
  K.MatVec(Kx.data(), 1.0, x.data(), 0.0);
  double rr = 0, bb = 0, xs = 0;
  for (size_t i = 0; i < b.size(); ++i) {
    rr += (b[i] - Kx[i]) * (b[i] - Kx[i]);
    bb += b[i] * b[i];
    xs += x[i];
  }
  // the same solve through the compatibility path (device vectors + ADL primitives)
  const size_t nd = b.size();
  g::DeviceVector dr(nd), dx(nd), dPr(nd), dp(nd);
  dr.upload(b.data());
  g::DeviceVectorView vr = dr.view(), vx = dx.view(), vPr = dPr.view(), vp = dp.view();
  const std::vector<double> hist2 = generic_pcg(vr, vx, vPr, vp, 1e-10, 1000, K, ilu);
  std::vector<double> x2(nd);
  dx.download(x2.data());
  double xs2 = 0;
  for (size_t i = 0; i < nd; ++i) xs2 += x2[i];
  std::printf("iterations %zu residual %.3e xsum %.17g compat_iterations %zu compat_xsum %.17g\n", hist.size() - 1,
              std::sqrt(rr / bb), xs, hist2.size() - 1, xs2);
  // the compatibility path's solution and history, for the caller to compare with the oracle
  if (argc > 2) {
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 4;
    const unsigned long long nh = hist2.size();
    std::fwrite(&nh, sizeof nh, 1, f);
    std::fwrite(hist2.data(), sizeof(double), hist2.size(), f);
    std::fwrite(x2.data(), sizeof(double), x2.size(), f);
    std::fclose(f);
  }
  return 0;
}

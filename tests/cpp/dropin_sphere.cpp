// The reference's hot-path call sequence (cluster tree, block-cluster tree,
// allocmbls, matgenGeH_omp, mltaGeHVec, mltaGeHhVec, subdivide_sym, matgenHeH_omp,
// mltaHeHVec, savembls, loadmbls, GMRes, freembls; with T = double and, for the
// Helmholtz kernel, T = dcomp) compiled against include/ahx_ahmed.hpp.  Checks
// the products against the dense matrices and GMRES on well-conditioned
// variants; exit status 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ahx_ahmed.hpp"

using namespace ahx_ahmed;

struct dof {
  double c[3];
  double getcenter(unsigned j) const { return c[j]; }
  double getradius2() const { return 0.0; }
};

// the MATGEN_T of this example: K = 1/(4 pi r), diagonal 1/(4 pi h)
struct LaplaceGen : LaplaceGenerator {
  explicit LaplaceGen(double hh) : LaplaceGenerator{hh} {}
};

// mblock<dcomp> leaves: exp(ikr)/(4 pi r), diagonal exp(ikh)/(4 pi h)
struct HelmholtzGen : HelmholtzGenerator {
  HelmholtzGen(double hh, double kk) : HelmholtzGenerator{hh, kk} {}
};

int main(int argc, char** argv) {
  const unsigned N = argc > 1 ? (unsigned)atoi(argv[1]) : 2048;
  const unsigned bmin = 32;
  const double eta = 0.8, eps = 1e-6;
  std::vector<dof> dofs(N);
  for (unsigned i = 0; i < N; ++i) {  // Fibonacci sphere
    const double z = 1.0 - 2.0 * (i + 0.5) / N, r = std::sqrt(1.0 - z * z);
    const double th = i * (M_PI * (3.0 - std::sqrt(5.0)));
    dofs[i].c[0] = r * std::cos(th);
    dofs[i].c[1] = r * std::sin(th);
    dofs[i].c[2] = z;
  }
  std::vector<double> pts(3 * (size_t)N);
  for (unsigned i = 0; i < N; ++i)
    for (int j = 0; j < 3; ++j) pts[3 * i + j] = dofs[i].c[j];
  const double h = ahx_mean_nn(pts.data(), N);

  std::vector<unsigned> op_perm(N), po_perm(N);
  for (unsigned i = 0; i < N; ++i) op_perm[i] = po_perm[i] = i;
  bemcluster<dof>* cl = new bemcluster<dof>(dofs.data(), op_perm.data(), 0, N);
  cl->createClusterTree(bmin, op_perm.data(), po_perm.data());
  unsigned nblcks = 0;
  bemblcluster<dof, dof>* bl = new bemblcluster<dof, dof>(0, 0, N, N);
  bl->subdivide(cl, cl, eta * eta, nblcks);
  std::printf("leaves %u admissible %lu\n", nblcks, bl->nadmleaves());
  if (argc > 2) {  // tree only (host): no device work
    delete bl;
    delete cl;
    return 0;
  }

  mblock<double>** A;
  allocmbls(bl, A);
  LaplaceGen gen{h};
  matgenGeH_omp(gen, nblcks, bl, eps, 1000000, A);
  unsigned lowrank = 0;
  for (unsigned l = 0; l < nblcks; ++l) lowrank += A[l]->isLrM();

  std::vector<double> x(N), y(N, 0.0);
  srand(1);
  for (unsigned i = 0; i < N; ++i) x[i] = 2.0 * rand() / RAND_MAX - 1.0;
  mltaGeHVec(1.0, bl, A, x.data(), y.data());
  std::vector<double> yt(N, 0.0);  // the kernel is symmetric: A^T x approximates the same
  mltaGeHhVec(1.0, bl, A, x.data(), yt.data());
  double num = 0.0, numt = 0.0, den = 0.0;
  for (unsigned i = 0; i < N; ++i) {  // dense product in the permuted ordering
    const dof& a = dofs[op_perm[i]];
    double s = 0.0;
    for (unsigned j = 0; j < N; ++j) {
      const dof& b = dofs[op_perm[j]];
      const double dx = a.c[0] - b.c[0], dy = a.c[1] - b.c[1], dz = a.c[2] - b.c[2];
      const double r = i == j ? h : std::sqrt(dx * dx + dy * dy + dz * dz);
      s += x[j] / (4.0 * M_PI * r);
    }
    num += (y[i] - s) * (y[i] - s);
    numt += (yt[i] - s) * (yt[i] - s);
    den += s * s;
  }
  const double err = std::sqrt(num / den), errt = std::sqrt(numt / den);
  std::printf("low-rank leaves %u, product error vs dense %.3e, adjoint %.3e\n", lowrank, err,
              errt);
  bool sym_ok = false;
  {  // the symmetric block tree, HeH assembly and product (Include/matgen_omp.h:96-101)
    unsigned nb = 0;
    bemblcluster<dof, dof>* bls = new bemblcluster<dof, dof>(0, 0, N, N);
    bls->subdivide_sym(cl, eta * eta, nb);
    mblock<double>** S;
    allocmbls(bls, S);
    matgenHeH_omp(gen, nb, bls, eps, 1000000, S);
    std::vector<double> ys(N, 0.0);
    mltaHeHVec(1.0, bls, S, x.data(), ys.data());
    double ds = 0.0, ns = 0.0;
    for (unsigned i = 0; i < N; ++i) {
      ds += (ys[i] - y[i]) * (ys[i] - y[i]);
      ns += y[i] * y[i];
    }
    unsigned hem = 0;
    for (unsigned l = 0; l < nb; ++l) hem += S[l]->isHeM();
    sym_ok = nb < nblcks && hem > 0 && std::sqrt(ds / ns) < 2e-6;
    std::printf("symmetric: %u leaves (%u Hermitian), product vs general %.3e\n", nb, hem, std::sqrt(ds / ns));
    freembls(bls, S);
    delete bls;
  }
  bool io_ok = false;
  {  // savembls -> loadmbls (Include/H.h:60-103) -> product on a tree built from the file
    {
      std::ofstream os("dropin_sphere.mbls", std::ios::binary);
      savembls(eta, bmin, bl, A, os);
    }
    double eta_f = 0.0;
    unsigned bmin_f = 0, nb = 0;
    mblock<double>** B = nullptr;
    std::ifstream is("dropin_sphere.mbls", std::ios::binary);
    loadmbls(eta_f, bmin_f, B, is);
    bemblcluster<dof, dof>* bl3 = new bemblcluster<dof, dof>(0, 0, N, N);
    bl3->subdivide(cl, cl, eta_f * eta_f, nb);
    std::vector<double> y3(N, 0.0);
    mltaGeHVec(1.0, bl3, B, x.data(), y3.data());
    double d3 = 0.0, n3 = 0.0;
    for (unsigned i = 0; i < N; ++i) {
      d3 += (y3[i] - y[i]) * (y3[i] - y[i]);
      n3 += y[i] * y[i];
    }
    io_ok = eta_f == eta && bmin_f == bmin && nb == nblcks && B[0]->getn1() == A[0]->getn1() &&
            std::sqrt(d3 / n3) < 1e-14;
    std::printf("savembls/loadmbls round trip %s\n", io_ok ? "ok" : "FAILED");
    freembls(bl3, B);
    delete bl3;
  }
  bool single_ok = false;
  {  // the single-precision instantiations: mblock<float> (FP32 leaves) and mblock<scomp>
    unsigned nb = 0;
    bemblcluster<dof, dof>* bls = new bemblcluster<dof, dof>(0, 0, N, N);
    bls->subdivide(cl, cl, eta * eta, nb);
    mblock<float>** F;
    allocmbls(bls, F);
    matgenGeH_omp(gen, nb, bls, eps, 1000000, F);
    std::vector<float> xf(x.begin(), x.end()), yf(N, 0.f);
    mltaGeHVec(1.0f, bls, F, xf.data(), yf.data());
    double df = 0.0, nf = 0.0;
    for (unsigned i = 0; i < N; ++i) {
      df += (yf[i] - y[i]) * (yf[i] - y[i]);
      nf += y[i] * y[i];
    }
    const bool f_ok = std::sqrt(df / nf) < 2e-6 && F[0]->getdata() != nullptr;
    freembls(bls, F);
    mblock<scomp>** C;
    allocmbls(bls, C);
    HelmholtzGen hg{h, 5.0};
    matgenGeH_omp(hg, nb, bls, eps, 1000000, C);
    mblock<dcomp>** Cd;  // the same leaves seen in double precision
    allocmbls(bls, Cd);
    for (unsigned l = 0; l < nb; ++l) Cd[l] = new mblock<dcomp>(bls, l);
    std::vector<scomp> xs(N), ys(N, 0.f);
    std::vector<dcomp> xd(N), yd(N, 0.0);
    for (unsigned i = 0; i < N; ++i) {
      xs[i] = scomp((float)x[i], (float)std::cos(0.1 * i));
      xd[i] = dcomp(xs[i].real(), xs[i].imag());
    }
    mltaGeHVec(scomp(1.f, 0.f), bls, C, xs.data(), ys.data());
    mltaGeHVec(dcomp(1.0, 0.0), bls, Cd, xd.data(), yd.data());
    double dc = 0.0, nc = 0.0;
    for (unsigned i = 0; i < N; ++i) {
      dc += std::norm(dcomp(ys[i].real(), ys[i].imag()) - yd[i]);
      nc += std::norm(yd[i]);
    }
    single_ok = f_ok && std::sqrt(dc / nc) < 2e-5 && C[0]->isLrM() == Cd[0]->isLrM();
    std::printf("single precision: float product error %.3e, scomp vs dcomp %.3e\n", std::sqrt(df / nf),
                std::sqrt(dc / nc));
    freembls(bls, Cd);
    freembls(bls, C);
    delete bls;
  }
  freembls(bl, A);
  delete bl;

  bool helm_ok = false;
  {  // the Helmholtz matrix with T = dcomp: assembly, A / A^H products, complex GMRes
    const double k = 5.0;
    unsigned nz = 0;
    bemblcluster<dof, dof>* blz = new bemblcluster<dof, dof>(0, 0, N, N);
    blz->subdivide(cl, cl, eta * eta, nz);
    mblock<dcomp>** Z;
    allocmbls(blz, Z);
    HelmholtzGen hg{h, k};
    matgenGeH_omp(hg, nz, blz, eps, 1000000, Z);
    unsigned zlr = 0;
    for (unsigned l = 0; l < nz; ++l) zlr += Z[l]->isLrM();
    std::vector<dcomp> zx(N), zy(N, 0.0), zyh(N, 0.0);
    for (unsigned i = 0; i < N; ++i) zx[i] = dcomp(x[i], std::cos(0.1 * i));
    mltaGeHVec(dcomp(1.0, 0.0), blz, Z, zx.data(), zy.data());
    mltaGeHhVec(dcomp(1.0, 0.0), blz, Z, zx.data(), zyh.data());
    double zn = 0.0, znh = 0.0, zd = 0.0, zdh = 0.0;
    for (unsigned i = 0; i < N; ++i) {  // dense A x and A^H x (A is complex symmetric)
      const dof& a = dofs[op_perm[i]];
      dcomp s = 0.0, sh = 0.0;
      for (unsigned j = 0; j < N; ++j) {
        const dof& b = dofs[op_perm[j]];
        const double dx = a.c[0] - b.c[0], dy = a.c[1] - b.c[1], dz = a.c[2] - b.c[2];
        const double r = i == j ? h : std::sqrt(dx * dx + dy * dy + dz * dz);
        const dcomp e = std::exp(dcomp(0.0, k * r)) / (4.0 * M_PI * r);
        s += e * zx[j];
        sh += std::conj(e) * zx[j];
      }
      zn += std::norm(zy[i] - s);
      znh += std::norm(zyh[i] - sh);
      zd += std::norm(s);
      zdh += std::norm(sh);
    }
    const double zerr = std::sqrt(zn / zd), zerrh = std::sqrt(znh / zdh);
    bool zio_ok = false;
    {  // savembls / loadmbls of the mblock<dcomp> leaves
      {
        std::ofstream os("dropin_helm.mbls", std::ios::binary);
        savembls(eta, bmin, blz, Z, os);
      }
      double eta_f = 0.0;
      unsigned bmin_f = 0, nb = 0;
      mblock<dcomp>** ZB = nullptr;
      std::ifstream is("dropin_helm.mbls", std::ios::binary);
      loadmbls(eta_f, bmin_f, ZB, is);
      bemblcluster<dof, dof>* bl4 = new bemblcluster<dof, dof>(0, 0, N, N);
      bl4->subdivide(cl, cl, eta_f * eta_f, nb);
      std::vector<dcomp> zy4(N, 0.0);
      mltaGeHVec(dcomp(1.0, 0.0), bl4, ZB, zx.data(), zy4.data());
      double d4 = 0.0, n4 = 0.0;
      for (unsigned i = 0; i < N; ++i) {
        d4 += std::norm(zy4[i] - zy[i]);
        n4 += std::norm(zy[i]);
      }
      zio_ok = nb == nz && ZB[0]->rank() == Z[0]->rank() && std::sqrt(d4 / n4) < 1e-14;
      freembls(bl4, ZB);
      delete bl4;
    }
    bool zaggl_ok = false;
    {  // agglH of the mblock<dcomp> leaves (H/agglH.cpp:291)
      const unsigned before = (unsigned)blz->nleaves();
      agglH(blz, Z, eps, 1000000);
      std::vector<dcomp> zy5(N, 0.0);
      mltaGeHVec(dcomp(1.0, 0.0), blz, Z, zx.data(), zy5.data());
      double d5 = 0.0, n5 = 0.0;
      for (unsigned i = 0; i < N; ++i) {
        d5 += std::norm(zy5[i] - zy[i]);
        n5 += std::norm(zy[i]);
      }
      zaggl_ok = blz->nleaves() < before && std::sqrt(d5 / n5) < 1e-5;
      std::printf("helmholtz agglH: %u -> %lu leaves, product change %.3e\n", before, blz->nleaves(),
                  std::sqrt(d5 / n5));
    }
    freembls(blz, Z);
    delete blz;
    // the complex symmetric form on the symmetric tree (matgenSyH_omp, mltaSyHVec)
    bemblcluster<dof, dof>* bls = new bemblcluster<dof, dof>(0, 0, N, N);
    unsigned ns = 0;
    bls->subdivide_sym(cl, eta * eta, ns);
    allocmbls(bls, Z);
    matgenSyH_omp(hg, ns, bls, eps, 1000000, Z);
    unsigned sym_diag = 0;
    for (unsigned l = 0; l < ns; ++l) sym_diag += Z[l]->isSyM();
    std::vector<dcomp> zys(N, 0.0);
    mltaSyHVec(dcomp(1.0, 0.0), bls, Z, zx.data(), zys.data());
    double zsd = 0.0, zsn = 0.0;
    for (unsigned i = 0; i < N; ++i) {
      zsd += std::norm(zys[i] - zy[i]);
      zsn += std::norm(zy[i]);
    }
    const double zserr = std::sqrt(zsd / zsn);
    freembls(bls, Z);
    delete bls;
    // complex GMRes with the diagonal of a well-conditioned variant (h_min / 8)
    bemblcluster<dof, dof>* blg = new bemblcluster<dof, dof>(0, 0, N, N);
    blg->subdivide(cl, cl, eta * eta, nz);
    allocmbls(blg, Z);
    HelmholtzGen hg2{ahx_min_nn(pts.data(), N) / 8.0, k};
    matgenGeH_omp(hg2, nz, blg, eps, 1000000, Z);
    ZHMatrixOperator zop(blg);
    std::vector<dcomp> zb(N), zs(N, 0.0);
    for (unsigned i = 0; i < N; ++i) zb[i] = dcomp(std::sin(0.37 * i), std::cos(0.11 * i));
    double zeps = 1e-8;
    unsigned zsteps = 300;
    const unsigned zret = GMRes(zop, zb.data(), zs.data(), zeps, 50, zsteps);
    freembls(blg, Z);
    delete blg;
    helm_ok = zlr > 0 && zerr < 5e-6 && zerrh < 5e-6 && zret == 0 && zeps < 1e-8 && sym_diag > 0 && zserr < 5e-6 &&
              zio_ok && zaggl_ok;
    std::printf("helmholtz: %u low-rank leaves, product error %.3e, adjoint %.3e, GMRes ret %u eps %.3e steps %u\n",
                zlr, zerr, zerrh, zret, zeps, zsteps);
    std::printf("helmholtz symmetric: %u leaves (%u symmetric diagonal), product vs general %.3e\n", ns, sym_diag,
                zserr);
    std::printf("helmholtz savembls/loadmbls round trip %s\n", zio_ok ? "ok" : "FAILED");
  }

  // GMRES on the SPD variant (diagonal 2/(4 pi h))
  bemblcluster<dof, dof>* bl2 = new bemblcluster<dof, dof>(0, 0, N, N);
  bl2->subdivide(cl, cl, eta * eta, nblcks);
  allocmbls(bl2, A);
  LaplaceGen gen2{h / 2.0};
  matgenGeH_omp(gen2, nblcks, bl2, eps, 1000000, A);
  HMatrixOperator op(bl2);
  std::vector<double> b(N), sol(N, 0.0);
  for (unsigned i = 0; i < N; ++i) b[i] = std::sin(0.37 * i);
  double geps = 1e-8;
  unsigned nsteps = 300;
  const unsigned ret = GMRes(op, b.data(), sol.data(), geps, 30, nsteps);
  std::printf("GMRes ret %u eps %.3e steps %u\n", ret, geps, nsteps);
  freembls(bl2, A);
  delete bl2;
  delete cl;
  return (err < 2e-6 && errt < 2e-6 && io_ok && sym_ok && helm_ok && single_ok && ret == 0 && geps < 1e-8) ? 0 : 1;
}

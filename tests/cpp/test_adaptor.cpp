// The reference's unit tests of the orbital hot path, written against the
// MGmol-shaped C++ surface of mgmol_adaptor.h and run on the GPU:
//   testLaph4 / testBatchLaph4 (tests/testLaph4.cc:7-86, testBatchLaph4.cc:7-110)
//   testMGkernels (tests/testMGkernels.cc:8-85)
//   testGramMatrix, single task (tests/testGramMatrix.cc:21-120)
// plus checks of Hamiltonian::applyLocal, OrbitalsPreconditioning, the
// residual / orbital update and pb::Mgm.
// Prints one line per check and exits non-zero on the first failure.
#include "mgmol_adaptor.h"

#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

static int failures = 0;
#define CHECK(cond, ...)                                                       \
    do                                                                         \
    {                                                                          \
        if (!(cond))                                                           \
        {                                                                      \
            std::printf("FAIL %s:%d ", __FILE__, __LINE__);                    \
            std::printf(__VA_ARGS__);                                          \
            std::printf("\n");                                                 \
            failures++;                                                        \
        }                                                                      \
    } while (0)

using namespace mgx;

static void sine_field(const pb::Grid& g, std::vector<double>& u, std::vector<double>& lap)
{
    const double k[3] = { 2 * M_PI / g.ll(0), 2 * M_PI / g.ll(1), 2 * M_PI / g.ll(2) };
    u.assign(g.size(), 0.);
    lap.assign(g.size(), 0.);
    for (unsigned x = 0; x < g.dim(0); x++)
        for (unsigned y = 0; y < g.dim(1); y++)
            for (unsigned z = 0; z < g.dim(2); z++)
            {
                const size_t i = ((size_t)x * g.dim(1) + y) * g.dim(2) + z;
                const double X = x * g.hgrid(0), Y = y * g.hgrid(1), Z = z * g.hgrid(2);
                u[i] = std::sin(k[0] * X) + std::sin(k[1] * Y) + std::sin(k[2] * Z);
                lap[i] = k[0] * k[0] * std::sin(k[0] * X) + k[1] * k[1] * std::sin(k[1] * Y)
                         + k[2] * k[2] * std::sin(k[2] * Z);
            }
}

static void test_laph4(int nfunc)
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 2., 2., 2. };
    const unsigned n[3] = { 32, 24, 20 };
    pb::Grid grid(origin, ll, n, 2);
    pb::Laph4<double> lap(grid);
    pb::GridFuncVector<double> gu(grid, nfunc), gv(grid, nfunc);
    std::vector<double> u, ex, out(grid.size());
    sine_field(grid, u, ex);
    for (int f = 0; f < nfunc; f++)
    {
        std::vector<double> uf(u);
        for (auto& x : uf) x *= (f + 1);
        gu.assign(f, uf.data());
    }
    lap.apply(gu, gv);
    for (int f = 0; f < nfunc; f++)
    {
        gv.getValues(f, out.data());
        double err = 0., mx = 0.;
        for (size_t i = 0; i < out.size(); i++)
        {
            err = std::max(err, std::fabs(out[i] - (f + 1) * ex[i]));
            mx  = std::max(mx, std::fabs((f + 1) * ex[i]));
        }
        CHECK(err < 2e-3 * mx, "Laph4 function %d: err %g", f, err / mx);
    }
    std::printf("ok   testLaph4 (nfunc = %d)\n", nfunc);
}

static void test_mgkernels()
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 3.2, 2.4, 2.0 };
    const unsigned n[3] = { 32, 24, 20 };
    pb::Grid fine(origin, ll, n, 1);
    pb::Grid coarse = fine.coarse_grid();
    pb::GridFuncVector<double> gf(fine, 5), gc(coarse, 5);
    for (int f = 0; f < 5; f++)
    {
        std::vector<double> c(fine.size(), f * 1.11);
        gf.assign(f, c.data());
    }
    gf.trade_boundaries();
    gf.restrict3D(gc);
    std::vector<double> vc(coarse.size()), vf(fine.size());
    for (int f = 0; f < 5; f++)
    {
        gc.getValues(f, vc.data());
        for (double v : vc) CHECK(std::fabs(v - f * 1.11) < 1e-8, "restrict %d: %g", f, v);
    }
    gc.set_updated_boundaries(false);
    gf.extend3D(gc);
    for (int f = 0; f < 5; f++)
    {
        gf.getValues(f, vf.data());
        for (double v : vf) CHECK(std::fabs(v - f * 1.11) < 1e-8, "extend %d: %g", f, v);
    }
    std::printf("ok   testMGkernels\n");
}

static void test_gram_matrix()
{
    const int n = 213;
    std::mt19937 gen(213);
    std::normal_distribution<double> N01;
    std::vector<double> A((size_t)n * n), S((size_t)n * n, 0.);
    for (auto& a : A) a = N01(gen);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            double s = 0.;
            for (int k = 0; k < n; k++) s += A[(size_t)i * n + k] * A[(size_t)j * n + k];
            S[(size_t)j * n + i] = s / n + (i == j ? 1. : 0.);
        }
    const double origin[3] = { 0, 0, 0 }, ll[3] = { 1, 1, 1 };
    const unsigned g8[3] = { 8, 8, 8 };
    pb::Grid grid(origin, ll, g8, 1);
    OrbitalBlock<double> dummy(grid, 1);
    GramMatrix gm(dummy.ctx(), n);
    DeviceArray<double> dS((size_t)n * n);
    dS.upload(S.data(), S.size());
    gm.setMatrix(dS);
    std::vector<double> L((size_t)n * n), Si((size_t)n * n);
    gm.getCholeskyL().download(L.data(), L.size());
    gm.getInverse().download(Si.data(), Si.size());
    double e1 = 0., e2 = 0., mx = 0.;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
        {
            double llt = 0., sis = 0.;
            for (int k = 0; k < n; k++)
            {
                llt += L[(size_t)k * n + i] * L[(size_t)k * n + j];
                sis += Si[(size_t)k * n + i] * S[(size_t)j * n + k];
            }
            e1 = std::max(e1, std::fabs(llt - S[(size_t)j * n + i]));
            e2 = std::max(e2, std::fabs(sis - (i == j ? 1. : 0.)));
            mx = std::max(mx, std::fabs(S[(size_t)j * n + i]));
        }
    CHECK(e1 <= 1e-14 * mx * n, "L L^T - S = %g", e1);
    CHECK(e2 < 1e-12, "S^-1 S - I = %g", e2);
    // a non-SPD matrix throws the status instead of aborting
    S[5 * n + 5] = -1.;
    dS.upload(S.data(), S.size());
    bool threw = false;
    try
    {
        gm.setMatrix(dS);
    }
    catch (const Error& e)
    {
        threw = (e.status == MGX_NOT_SPD);
    }
    CHECK(threw, "non-SPD matrix not reported");
    std::printf("ok   testGramMatrix (one task)\n");
}

static void test_hamiltonian_and_precond()
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 6.4, 6.4, 6.4 };
    const unsigned n[3] = { 32, 32, 32 };
    pb::Grid grid(origin, ll, n, 1);
    const int nf = 3;
    OrbitalBlock<double> phi(grid, nf), hphi(grid, nf);
    std::vector<double> u, ex, all;
    sine_field(grid, u, ex);
    for (int f = 0; f < nf; f++) all.insert(all.end(), u.begin(), u.end());
    phi.set(all.data());
    DeviceArray<double> V(grid.size()); // zero potential: H phi = -Lap_M phi
    Hamiltonian<double> H(0);
    H.applyLocal(phi, V, hphi);
    std::vector<double> out(all.size());
    hphi.get(out.data());
    double err = 0., mx = 0.;
    for (size_t i = 0; i < u.size(); i++)
    {
        err = std::max(err, std::fabs(out[i] - ex[i]));
        mx  = std::max(mx, std::fabs(ex[i]));
    }
    // -Lap_M u approximates B(-Lap u); B differs from 1 by O(h^2 k^2)
    CHECK(err < 5e-2 * mx, "Mehrstellen H phi vs -Lap phi: %g", err / mx);
    // the preconditioner is linear: P(2 r) = 2 P(r)
    OrbitalsPreconditioning<double> P;
    P.setup(2, 0);
    P.setGamma(grid, 0.0, -1.0);
    OrbitalBlock<double> r1(grid, nf), r2(grid, nf);
    std::vector<double> two(all);
    for (auto& x : two) x *= 2.;
    r1.set(all.data());
    r2.set(two.data());
    P.precond_mg(r1);
    P.precond_mg(r2);
    std::vector<double> a(all.size()), b(all.size());
    r1.get(a.data());
    r2.get(b.data());
    double lin = 0., am = 0.;
    for (size_t i = 0; i < a.size(); i++)
    {
        lin = std::max(lin, std::fabs(b[i] - 2. * a[i]));
        am  = std::max(am, std::fabs(a[i]));
    }
    CHECK(am > 0. && lin < 1e-12 * am, "precond linearity %g", lin / am);
    // S of identical orbitals: every entry equals the squared norm
    DeviceArray<double> S((size_t)nf * nf);
    phi.computeGram(S);
    std::vector<double> hs((size_t)nf * nf);
    S.download(hs.data(), hs.size());
    double nrm = 0.;
    for (double x : u) nrm += x * x;
    nrm *= grid.vel();
    for (double s : hs) CHECK(std::fabs(s - nrm) < 1e-12 * nrm, "Gram entry %g vs %g", s, nrm);
    std::printf("ok   Hamiltonian::applyLocal, OrbitalsPreconditioning, computeGram\n");
}

/* computeResidualUsingHPhi without B and with theta = 2 I: res = 2 phi -
 * hphi; then pb::Mgm with Laph2 on one sine mode, whose discrete solution
 * is rho / lambda, lambda = (2 - 2 cos(k h)) / h^2. */
static void test_residual_and_mgm()
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 6.4, 4.8, 8.0 };
    const unsigned n[3] = { 32, 24, 40 };
    pb::Grid grid(origin, ll, n, 1);
    const int nf = 3;
    OrbitalBlock<double> phi(grid, nf), hphi(grid, nf), res(grid, nf);
    std::vector<double> u, ex, all;
    sine_field(grid, u, ex);
    for (int f = 0; f < nf; f++)
        for (double x : u) all.push_back((f + 1) * x);
    phi.set(all.data());
    std::vector<double> hp(all.size());
    for (size_t i = 0; i < hp.size(); i++) hp[i] = 0.25 * all[i] + 1.;
    hphi.set(hp.data());
    std::vector<double> th((size_t)nf * nf, 0.);
    for (int i = 0; i < nf; i++) th[(size_t)i * nf + i] = 2.;
    DeviceArray<double> theta(th.size());
    theta.upload(th.data(), th.size());
    computeResidualUsingHPhi(phi, hphi, theta, res, false);
    std::vector<double> r(all.size());
    res.get(r.data());
    double err = 0.;
    for (size_t i = 0; i < r.size(); i++) err = std::max(err, std::fabs(r[i] - (2. * all[i] - hp[i])));
    CHECK(err < 1e-13, "residual without B: %g", err);
    // multiplyByMatrix with the same theta doubles the block, then axpy undoes it
    phi.multiplyByMatrix(theta, res);
    res.axpy(-1., phi);
    res.get(r.data());
    err = 0.;
    for (size_t i = 0; i < r.size(); i++) err = std::max(err, std::fabs(r[i] - all[i]));
    CHECK(err < 1e-13, "multiplyByMatrix / axpy: %g", err);

    const double kx = 2 * M_PI / ll[0], h = grid.hgrid(0);
    const double lambda = (2. - 2. * std::cos(kx * h)) / (h * h);
    std::vector<double> rho(grid.size()), exact(grid.size());
    for (unsigned x = 0; x < n[0]; x++)
        for (unsigned y = 0; y < n[1]; y++)
            for (unsigned z = 0; z < n[2]; z++)
            {
                const size_t i = ((size_t)x * n[1] + y) * n[2] + z;
                rho[i]   = std::sin(kx * x * h);
                exact[i] = rho[i] / lambda;
            }
    DeviceArray<double> vh(grid.size()), drho(grid.size());
    drho.upload(rho.data(), rho.size());
    pb::Laph2<double> A(grid);
    double fr = 0., frr = 0., red = 0.;
    short nb  = 0;
    const bool conv = pb::Mgm(A, grid, vh.data(), drho.data(), 10, 30, 1e-11, 2, 2, false, fr,
        frr, red, nb);
    std::vector<double> sol(grid.size());
    vh.download(sol.data(), sol.size());
    double e2 = 0., m2 = 0.;
    for (size_t i = 0; i < sol.size(); i++)
    {
        e2 = std::max(e2, std::fabs(sol[i] - exact[i]));
        m2 = std::max(m2, std::fabs(exact[i]));
    }
    CHECK(conv && frr < 1e-11 && nb > 0, "Mgm converged %d, rel %g, sweeps %d", (int)conv, frr, nb);
    CHECK(e2 < 1e-9 * m2, "Mgm vs the discrete solution: %g", e2 / m2);
    std::printf("ok   computeResidualUsingHPhi, multiplyByMatrix, pb::Mgm (%d V-cycles)\n", nb);
}

/* LocGridOrbitals::normalize, computeMatB and ProjectedMatricesMehrstellen
 * on three plane waves along x, sin(kx), sin(2kx), cos(kx): the
 * Mehrstellen right-hand side acts on a wave of wave number q as
 * 5/6 + cos(q h)/6, so after normalization B is diagonal with those
 * entries, invB their inverses, theta = invB H for diagonal H, and
 * HB = theta for S = I. */
static void test_matb_normalize()
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 6.4, 4.8, 8.0 };
    const unsigned n[3] = { 32, 24, 40 };
    pb::Grid grid(origin, ll, n, 1);
    const int nf = 3;
    OrbitalBlock<double> phi(grid, nf);
    const double kx = 2 * M_PI / ll[0], h = grid.hgrid(0);
    const double q[nf] = { kx, 2 * kx, kx };
    std::vector<double> all((size_t)nf * grid.size());
    for (int f = 0; f < nf; f++)
        for (unsigned x = 0; x < n[0]; x++)
            for (unsigned yz = 0; yz < n[1] * n[2]; yz++)
                all[(size_t)f * grid.size() + (size_t)x * n[1] * n[2] + yz]
                    = (f + 2.) * (f == 2 ? std::cos(q[f] * x * h) : std::sin(q[f] * x * h));
    phi.set(all.data());
    phi.normalize();
    std::vector<double> u(all.size());
    phi.get(u.data());
    for (int f = 0; f < nf; f++)
    {
        double s2 = 0.;
        for (size_t i = 0; i < grid.size(); i++)
            s2 += u[(size_t)f * grid.size() + i] * u[(size_t)f * grid.size() + i];
        CHECK(std::fabs(s2 * grid.vel() - 1.) < 1e-12, "normalize: vel |psi|^2 = %.16g", s2 * grid.vel());
    }
    DeviceArray<double> B((size_t)nf * nf);
    phi.computeMatB(B);
    std::vector<double> hb((size_t)nf * nf);
    B.download(hb.data(), hb.size());
    double mu[nf];
    for (int f = 0; f < nf; f++)
        mu[f] = 5. / 6. + std::cos(q[f] * h) / 6.;
    double err = 0.;
    for (int j = 0; j < nf; j++)
        for (int i = 0; i < nf; i++)
            err = std::max(err, std::fabs(hb[(size_t)j * nf + i] - (i == j ? mu[i] : 0.)));
    CHECK(err < 1e-13, "computeMatB vs 5/6 + cos(qh)/6: %g", err);
    ProjectedMatricesMehrstellen pm(phi.ctx(), nf);
    pm.initializeMatB(B);
    pm.computeInvB();
    std::vector<double> hd((size_t)nf * nf, 0.), id((size_t)nf * nf, 0.);
    const double eps[nf] = { -0.5, 0.25, 1.5 };
    for (int i = 0; i < nf; i++)
    {
        hd[(size_t)i * nf + i] = eps[i];
        id[(size_t)i * nf + i] = 1.;
    }
    DeviceArray<double> H(hd.size()), S(id.size()), theta(hd.size()), HB(hd.size());
    H.upload(hd.data(), hd.size());
    S.upload(id.data(), id.size());
    pm.updateTheta(H, theta);
    pm.updateHB(S, theta, HB);
    std::vector<double> th(hd.size()), hbm(hd.size()), ib(hd.size());
    theta.download(th.data(), th.size());
    HB.download(hbm.data(), hbm.size());
    pm.getInvB().download(ib.data(), ib.size());
    err = 0.;
    for (int j = 0; j < nf; j++)
        for (int i = 0; i < nf; i++)
        {
            const double t = i == j ? eps[i] / mu[i] : 0.;
            err = std::max(err, std::fabs(th[(size_t)j * nf + i] - t));
            err = std::max(err, std::fabs(hbm[(size_t)j * nf + i] - t));
            err = std::max(err, std::fabs(ib[(size_t)j * nf + i] - (i == j ? 1. / mu[i] : 0.)));
        }
    CHECK(err < 1e-13, "computeInvB / updateTheta / updateHB: %g", err);
    // Rho with the density matrix X = 2 I on the normalized waves: rho =
    // 2 sum_f psi_f^2, whose charge is 2 nf
    DeviceArray<double> X(hd.size());
    std::vector<double> x2((size_t)nf * nf, 0.);
    for (int i = 0; i < nf; i++)
        x2[(size_t)i * nf + i] = 2.;
    X.upload(x2.data(), x2.size());
    Rho<double> rho(grid);
    const double charge = rho.computeRho(phi, X, 2. * nf);
    CHECK(std::fabs(charge - 2. * nf) < 1e-12, "Rho charge %.16g", charge);
    std::vector<double> r(grid.size());
    rho.rho().download(r.data(), r.size());
    err = 0.;
    for (size_t p = 0; p < grid.size(); p++)
    {
        double s2 = 0.;
        for (int f = 0; f < nf; f++)
            s2 += 2. * u[(size_t)f * grid.size() + p] * u[(size_t)f * grid.size() + p];
        err = std::max(err, std::fabs(r[p] - s2));
    }
    CHECK(err < 1e-13, "Rho vs 2 sum psi^2: %g", err);
    std::printf("ok   normalize, computeMatB, ProjectedMatricesMehrstellen, Rho\n");
}

/* SpreadsAndCenters: Gaussian orbitals (periodic images summed) put their
 * centre where they were placed; the spread is the periodic formula
 * sum_d (1 - exp(-k_d^2 s2)) / k_d^2 with s2 = sigma^2 / 2 */
static void test_spreads_and_centers()
{
    const double origin[3] = { 0., 0., 0. }, ll[3] = { 12.8, 11.2, 9.6 };
    const unsigned n[3] = { 40, 36, 32 };
    pb::Grid grid(origin, ll, n, 1);
    const int nf = 3;
    const double c[nf][3] = { { 1.1, 10.9, 4.0 }, { 6.4, 5.6, 9.5 }, { 12.2, 0.3, 0.05 } };
    const double sig = 1.0;
    OrbitalBlock<double> phi(grid, nf);
    std::vector<double> all((size_t)nf * grid.size());
    const double h[3] = { grid.hgrid(0), grid.hgrid(1), grid.hgrid(2) };
    for (int f = 0; f < nf; f++)
        for (unsigned x = 0; x < n[0]; x++)
            for (unsigned y = 0; y < n[1]; y++)
                for (unsigned z = 0; z < n[2]; z++)
                {
                    double v = 1.;
                    const unsigned idx[3] = { x, y, z };
                    for (int d = 0; d < 3; d++)
                    {
                        double g = 0.;
                        for (int img = -2; img <= 2; img++)
                        {
                            const double t = idx[d] * h[d] - c[f][d] + img * ll[d];
                            g += std::exp(-t * t / (2 * sig * sig));
                        }
                        v *= g;
                    }
                    all[(size_t)f * grid.size() + ((size_t)x * n[1] + y) * n[2] + z] = v;
                }
    phi.set(all.data());
    SpreadsAndCenters<double> sc(grid);
    sc.computePositionMatrix(phi);
    double err = 0., serr = 0.;
    double expect = 0.;
    for (int d = 0; d < 3; d++)
    {
        const double k = 2 * M_PI / ll[d];
        expect += (1. - std::exp(-k * k * sig * sig / 2)) / (k * k);
    }
    for (int f = 0; f < nf; f++)
    {
        const auto x = sc.computeCenter(f);
        for (int d = 0; d < 3; d++)
        {
            double dd = x[d] - c[f][d];
            dd -= ll[d] * std::round(dd / ll[d]);
            err = std::max(err, std::fabs(dd));
        }
        serr = std::max(serr, std::fabs(sc.computeSpread2(f) - expect));
    }
    CHECK(err < 1e-6, "SpreadsAndCenters centre error %g", err);
    CHECK(serr < 1e-5, "SpreadsAndCenters spread^2 error %g", serr);
    std::printf("ok   SpreadsAndCenters\n");
}

int main()
{
    try
    {
        test_laph4(1);
        test_laph4(10);
        test_mgkernels();
        test_gram_matrix();
        test_hamiltonian_and_precond();
        test_residual_and_mgm();
        test_matb_normalize();
        test_spreads_and_centers();
    }
    catch (const std::exception& e)
    {
        std::printf("FAIL exception: %s\n", e.what());
        return 2;
    }
    return failures ? 1 : 0;
}

/*
 * CPU oracle for the pychem Hartree-Fock integral path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the integral algorithm of the upstream reference
 * (dlc62/pychem).  It is linked only by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg, always as the checker; the library never calls it.
 *
 * What it follows (reference paths):
 *   pair data ........ Methods/c_ints/shellpair_quantities.c:5-38
 *                      sigma = 1/(a+b), U = (pi sigma)^{3/2} exp(-ab sigma |A-B|^2),
 *                      P = (aA + bB) sigma
 *   normalisation .... Util/structures.py:843,850-856 (ScaledCCs = cc (2a)^{(l+1.5)/2},
 *                      ContractionScaling = (G(lx+.5)G(ly+.5)G(lz+.5))^{-1/2});
 *                      contracted functions are NOT renormalised (as upstream)
 *   Cartesian order .. Methods/c_ints/angmom_index.c:3-15 (lx descending, then ly)
 *   Boys F_m(T) ...... Methods/c_ints/two_electron_fundamentals.c:6-95 evaluates F_m
 *                      from a table; here F_m is evaluated from its convergent series
 *                      plus downward recursion, accurate to a few ulp
 *   1e integrals ..... Methods/integrals.py:220-370 with one_electron_{fundamentals,
 *                      vrr,hrr,kinetic,contract}.c: Obara-Saika overlap and nuclear
 *                      attraction recurrences, kinetic energy from overlaps
 *                      [a|b+2], [a|b], [a|b-2] (one_electron_kinetic.c:60-64)
 *   2e integrals ..... Methods/integrals.py:427-555: Head-Gordon-Pople scheme -- VRR
 *                      on primitives to [e0|f0] (two_electron_vrr.c:92-109, written
 *                      here in the standard unscaled Obara-Saika form), contraction
 *                      (two_electron_contract.c:45), bra and ket HRR on contracted
 *                      integrals (two_electron_hrr.c:82), Cartesian normalisation and
 *                      Cartesian->spherical transform (integrals.py:541-547)
 *   scattering ....... Methods/c_ints/two_electron_scattering.c:6-81 (the j0(S r12)
 *                      operator of Methods/properties.py: fundamentals
 *                      U_P U_Q exp(-S^2 (sigma_P + sigma_Q)/4) S^2m z^-m j_m(z),
 *                      z = S |P - Q|, with its S = 0 and R = 0 cases), written here in
 *                      the unscaled Obara-Saika form (an extra (2 rho)^-m); z^-m j_m
 *                      by the piecewise scheme of spherical_bessel_j.c:5-81
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OR_MAXL 2             /* shells up to d */
#define OR_MAXLT (4 * OR_MAXL)
#define OR_MAXPRIM 16

typedef struct {
    int l, nprim;
    double center[3];
    double exps[OR_MAXPRIM];
    double ccs[OR_MAXPRIM]; /* raw contraction coefficients from the basis library */
} or_shell;

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int cart_offset(int l) { return l * (l + 1) * (l + 2) / 6; }
static int cart_index(int lx, int ly, int lz) { int s = ly + lz; return s * (s + 1) / 2 + lz; }
static int gidx(int lx, int ly, int lz) { return cart_offset(lx + ly + lz) + cart_index(lx, ly, lz); }

/* F_m(T), m = 0..mmax: for T < 30 the positive series for the top order, then
 * downward recursion; for T >= 30, F_0 = sqrt(pi/T) erf(sqrt T) / 2 and the upward
 * recursion F_{m+1} = ((2m+1) F_m - exp(-T)) / (2T), which is stable there. */
void oracle_boys(int mmax, double T, double *F)
{
    double e = exp(-T);
    if (T >= 30.0) {
        F[0] = 0.5 * sqrt(M_PI / T) * erf(sqrt(T));
        for (int m = 0; m < mmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * T);
        return;
    }
    double term = 1.0 / (2 * mmax + 1), acc = term;
    for (int k = 1; k < 4000; ++k) {
        term *= 2.0 * T / (2 * mmax + 2 * k + 1);
        acc += term;
        if (k > 10 && term < 1e-18 * acc) break;
    }
    F[mmax] = e * acc;
    for (int m = mmax; m > 0; --m) F[m - 1] = (2.0 * T * F[m] + e) / (2 * m - 1);
}

/* Normalised contraction coefficient of primitive k (ScaledCCs, structures.py:843). */
static double scaled_cc(const or_shell *s, int k)
{
    return s->ccs[k] * pow(2.0 * s->exps[k], (s->l + 1.5) / 2.0);
}

/* Per-component Cartesian normalisation (ContractionScaling, structures.py:850-856). */
static double comp_scale(int lx, int ly, int lz)
{
    return 1.0 / sqrt(tgamma(lx + 0.5) * tgamma(ly + 0.5) * tgamma(lz + 0.5));
}

/* Cartesian -> spherical rows (Data/transform_basis.py:3-12, Python 3 semantics). */
static void c2s_matrix(int l, double *M /* (2l+1) x ncart(l) */)
{
    int nc = ncart(l);
    memset(M, 0, sizeof(double) * (2 * l + 1) * nc);
    if (l == 0) { M[0] = 1.0; return; }
    if (l == 1) { for (int i = 0; i < 3; ++i) M[i * 3 + i] = 1.0; return; }
    /* d: xx xy xz yy yz zz */
    double h = sqrt(3.0) / 2.0;
    M[0 * 6 + 0] = h;  M[0 * 6 + 3] = -h;
    M[1 * 6 + 1] = 1.0;
    M[2 * 6 + 2] = 1.0;
    M[3 * 6 + 4] = 1.0;
    M[4 * 6 + 0] = -0.5; M[4 * 6 + 3] = -0.5; M[4 * 6 + 5] = 1.0;
}

static void list_cart(int l, int (*c)[3])
{
    int k = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) { c[k][0] = lx; c[k][1] = ly; c[k][2] = l - lx - ly; ++k; }
}

/* Apply the per-component scaling and the Cartesian->spherical transform to a block
 * cart[(ia,ib,ic,id)] laid out row-major over ncart of each shell; nshell = 2 or 4. */
static void to_spherical(int nshell, const int *ls, const double *cart, double *out)
{
    double buf0[1296], buf1[1296];
    int nc[4], ns[4];
    for (int s = 0; s < nshell; ++s) { nc[s] = ncart(ls[s]); ns[s] = 2 * ls[s] + 1; }
    int total = 1;
    for (int s = 0; s < nshell; ++s) total *= nc[s];
    memcpy(buf0, cart, sizeof(double) * total);
    /* scaling */
    {
        int comps[4][15][3];
        for (int s = 0; s < nshell; ++s) list_cart(ls[s], comps[s]);
        int idx[4] = {0, 0, 0, 0};
        for (int t = 0; t < total; ++t) {
            int r = t;
            for (int s = nshell - 1; s >= 0; --s) { idx[s] = r % nc[s]; r /= nc[s]; }
            double f = 1.0;
            for (int s = 0; s < nshell; ++s)
                f *= comp_scale(comps[s][idx[s]][0], comps[s][idx[s]][1], comps[s][idx[s]][2]);
            buf0[t] *= f;
        }
    }
    /* transform one index at a time: dims d[0..n-1], replace dim s by ns[s] */
    int dims[4];
    for (int s = 0; s < nshell; ++s) dims[s] = nc[s];
    double *src = buf0, *dst = buf1;
    for (int s = 0; s < nshell; ++s) {
        double M[5 * 6];
        c2s_matrix(ls[s], M);
        int outer = 1, inner = 1;
        for (int q = 0; q < s; ++q) outer *= dims[q];
        for (int q = s + 1; q < nshell; ++q) inner *= dims[q];
        for (int o = 0; o < outer; ++o)
            for (int i = 0; i < ns[s]; ++i)
                for (int n = 0; n < inner; ++n) {
                    double acc = 0.0;
                    for (int c = 0; c < nc[s]; ++c)
                        acc += M[i * nc[s] + c] * src[(o * nc[s] + c) * inner + n];
                    dst[(o * ns[s] + i) * inner + n] = acc;
                }
        dims[s] = ns[s];
        double *t = src; src = dst; dst = t;
    }
    int nout = 1;
    for (int s = 0; s < nshell; ++s) nout *= ns[s];
    memcpy(out, src, sizeof(double) * nout);
}

/* ------------------------------------------------------------------------------- */
/* One-electron integrals                                                           */
/* ------------------------------------------------------------------------------- */

/* 1D overlap factors E[i][j] for i <= imax, j <= jmax (Obara-Saika). */
static void overlap_1d(int imax, int jmax, double PA, double PB, double oo2z, double E[8][8])
{
    E[0][0] = 1.0;
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j <= jmax; ++j) {
            if (i == 0 && j == 0) continue;
            double v;
            if (j == 0) {
                v = PA * E[i - 1][0];
                if (i > 1) v += (i - 1) * oo2z * E[i - 2][0];
            } else {
                v = PB * E[i][j - 1];
                if (i > 0) v += i * oo2z * E[i - 1][j - 1];
                if (j > 1) v += (j - 1) * oo2z * E[i][j - 2];
            }
            E[i][j] = v;
        }
}

/* Nuclear attraction over primitives via Obara-Saika on a (a|V^(m)|b) table. */
static void nuclear_prim(int la, int lb, const double *A, const double *B, double alpha, double beta,
                         const double *C, double Z, double U, double *out /* ncart(la)*ncart(lb) */)
{
    int L = la + lb;
    double zeta = alpha + beta, oo2z = 0.5 / zeta;
    double P[3], PA[3], PB[3], PC[3], r2 = 0.0;
    for (int i = 0; i < 3; ++i) {
        P[i] = (alpha * A[i] + beta * B[i]) / zeta;
        PA[i] = P[i] - A[i]; PB[i] = P[i] - B[i]; PC[i] = P[i] - C[i];
        r2 += PC[i] * PC[i];
    }
    double F[OR_MAXLT + 2];
    oracle_boys(L, zeta * r2, F);
    /* table V[ga][gb][m] */
    static __thread double V[35][35][OR_MAXLT + 2];
    int na = cart_offset(la + 1), nb = cart_offset(lb + 1);
    double pre = -Z * 2.0 * sqrt(zeta / M_PI) * U; /* = -Z 2pi/zeta K_AB */
    for (int m = 0; m <= L; ++m) V[0][0][m] = pre * F[m];
    /* build a with b = 0 */
    for (int l = 1; l <= la; ++l) {
        int comps[15][3]; list_cart(l, comps);
        for (int k = 0; k < ncart(l); ++k) {
            int a[3] = {comps[k][0], comps[k][1], comps[k][2]};
            int i = a[0] ? 0 : (a[1] ? 1 : 2);
            int am[3] = {a[0], a[1], a[2]}; am[i]--;
            int g = gidx(a[0], a[1], a[2]), g1 = gidx(am[0], am[1], am[2]);
            int g2 = -1;
            if (am[i] > 0) { int amm[3] = {am[0], am[1], am[2]}; amm[i]--; g2 = gidx(amm[0], amm[1], amm[2]); }
            for (int m = 0; m <= L - l; ++m) {
                double v = PA[i] * V[g1][0][m] - PC[i] * V[g1][0][m + 1];
                if (g2 >= 0) v += am[i] * oo2z * (V[g2][0][m] - V[g2][0][m + 1]);
                V[g][0][m] = v;
            }
        }
    }
    /* build b for every a <= la */
    for (int lbb = 1; lbb <= lb; ++lbb) {
        int bcomps[15][3]; list_cart(lbb, bcomps);
        for (int kb = 0; kb < ncart(lbb); ++kb) {
            int b[3] = {bcomps[kb][0], bcomps[kb][1], bcomps[kb][2]};
            int i = b[0] ? 0 : (b[1] ? 1 : 2);
            int bm[3] = {b[0], b[1], b[2]}; bm[i]--;
            int gb = gidx(b[0], b[1], b[2]), gb1 = gidx(bm[0], bm[1], bm[2]);
            int gb2 = -1;
            if (bm[i] > 0) { int bmm[3] = {bm[0], bm[1], bm[2]}; bmm[i]--; gb2 = gidx(bmm[0], bmm[1], bmm[2]); }
            for (int laa = 0; laa <= la; ++laa) {
                int acomps[15][3]; list_cart(laa, acomps);
                for (int ka = 0; ka < ncart(laa); ++ka) {
                    int a[3] = {acomps[ka][0], acomps[ka][1], acomps[ka][2]};
                    int ga = gidx(a[0], a[1], a[2]);
                    int ga1 = -1;
                    if (a[i] > 0) { int am[3] = {a[0], a[1], a[2]}; am[i]--; ga1 = gidx(am[0], am[1], am[2]); }
                    for (int m = 0; m <= L - laa - lbb; ++m) {
                        double v = PB[i] * V[ga][gb1][m] - PC[i] * V[ga][gb1][m + 1];
                        if (ga1 >= 0) v += a[i] * oo2z * (V[ga1][gb1][m] - V[ga1][gb1][m + 1]);
                        if (gb2 >= 0) v += bm[i] * oo2z * (V[ga][gb2][m] - V[ga][gb2][m + 1]);
                        V[ga][gb][m] = v;
                    }
                }
            }
        }
    }
    (void)na; (void)nb;
    int ac[15][3], bc[15][3];
    list_cart(la, ac); list_cart(lb, bc);
    for (int ka = 0; ka < ncart(la); ++ka)
        for (int kb = 0; kb < ncart(lb); ++kb)
            out[ka * ncart(lb) + kb] = V[gidx(ac[ka][0], ac[ka][1], ac[ka][2])][gidx(bc[kb][0], bc[kb][1], bc[kb][2])][0];
}

/* S, T and V(all nuclei) for one shell pair, spherical, (2la+1) x (2lb+1) each.
 * nuc_xyz: natom x 3 (bohr), nuc_z: natom charges. */
int oracle_one_electron(const or_shell *sa, const or_shell *sb, int natom, const double *nuc_xyz,
                        const double *nuc_z, double *S_out, double *T_out, double *V_out)
{
    int la = sa->l, lb = sb->l, nca = ncart(la), ncb = ncart(lb);
    double Sc[36] = {0}, Tc[36] = {0}, Vc[36] = {0};
    int ac[15][3], bc[15][3];
    list_cart(la, ac); list_cart(lb, bc);
    const double *A = sa->center, *B = sb->center;
    double AB2 = 0.0;
    for (int i = 0; i < 3; ++i) AB2 += (A[i] - B[i]) * (A[i] - B[i]);
    for (int p = 0; p < sa->nprim; ++p)
        for (int q = 0; q < sb->nprim; ++q) {
            double a = sa->exps[p], b = sb->exps[q], zeta = a + b, sigma = 1.0 / zeta;
            double U = pow(M_PI * sigma, 1.5) * exp(-a * b * sigma * AB2);
            double cc = scaled_cc(sa, p) * scaled_cc(sb, q);
            double E[3][8][8];
            for (int i = 0; i < 3; ++i) {
                double P = (a * A[i] + b * B[i]) * sigma;
                overlap_1d(la, lb + 2, P - A[i], P - B[i], 0.5 * sigma, E[i]);
            }
            for (int ka = 0; ka < nca; ++ka)
                for (int kb = 0; kb < ncb; ++kb) {
                    const int *x = ac[ka], *y = bc[kb];
                    double s = E[0][x[0]][y[0]] * E[1][x[1]][y[1]] * E[2][x[2]][y[2]];
                    /* kinetic from overlaps (one_electron_kinetic.c:60-64) */
                    double t = b * (2 * lb + 3) * s;
                    for (int i = 0; i < 3; ++i) {
                        int yp[3] = {y[0], y[1], y[2]}; yp[i] += 2;
                        t -= 2.0 * b * b * E[0][x[0]][yp[0]] * E[1][x[1]][yp[1]] * E[2][x[2]][yp[2]];
                        if (y[i] > 1) {
                            int ym[3] = {y[0], y[1], y[2]}; ym[i] -= 2;
                            t -= 0.5 * y[i] * (y[i] - 1) * E[0][x[0]][ym[0]] * E[1][x[1]][ym[1]] * E[2][x[2]][ym[2]];
                        }
                    }
                    Sc[ka * ncb + kb] += cc * U * s;
                    Tc[ka * ncb + kb] += cc * U * t;
                }
            for (int c = 0; c < natom; ++c) {
                double v[36];
                nuclear_prim(la, lb, A, B, a, b, nuc_xyz + 3 * c, nuc_z[c], U, v);
                for (int k = 0; k < nca * ncb; ++k) Vc[k] += cc * v[k];
            }
        }
    int ls[2] = {la, lb};
    to_spherical(2, ls, Sc, S_out);
    to_spherical(2, ls, Tc, T_out);
    to_spherical(2, ls, Vc, V_out);
    return 0;
}

/* ------------------------------------------------------------------------------- */
/* Two-electron repulsion integrals, HGP                                            */
/* ------------------------------------------------------------------------------- */

#define NE_MAX 35 /* cart_offset(5): all Cartesians with l <= 4 */

/* Two-electron operator: 0 = 1/r12, 1 = j0(S r12) (electron scattering). */
static int g_op = 0;
static double g_S = 0.0;

void oracle_set_operator(int op, double S) { g_op = op; g_S = S; }

/* z^-m j_m(z), m = 0..lmax, by the regimes of spherical_bessel_j.c: the power series
 * about 0 below z = 10 (1, 3, 6 or 20 terms by the size of z), the two-term
 * asymptotic form above 100, upward recursion from j0 and j1 between; values below
 * 1e-16 in magnitude set to 0. */
void oracle_sph_bessel(int lmax, double z, double *j)
{
    if (z < 10.0) {
        int kmax = z < 1e-3 ? 1 : (z < 1e-1 ? 3 : (z < 1.0 ? 6 : 20));
        double z2 = z * z, df = 1.0;
        for (int m = 0; m <= lmax; ++m) {
            df *= (double)(2 * m + 1);
            double sum = 1.0, odd = (double)(2 * m + 1), oddprod = 1.0, zp = 1.0, den = 1.0, sg = 1.0;
            for (int k = 1; k <= kmax; ++k) {
                odd += 2.0;
                oddprod *= odd;
                zp *= z2;
                sg = -sg;
                den *= 2.0 * k;
                sum += sg * zp / (den * oddprod);
            }
            j[m] = sum / df;
        }
    } else if (z > 100.0) {
        double zi = 1.0 / z, zi2 = zi * zi, zm = 1.0, shift = z;
        j[0] = sin(z) * zi;
        for (int m = 1; m <= lmax; ++m) {
            double c = (double)(m * (m + 1) / 2);
            zm *= zi;
            shift -= 0.5 * M_PI;
            j[m] = zm * (zi * sin(shift) + c * zi2 * cos(shift));
        }
    } else {
        double zi = 1.0 / z, r[17];
        r[0] = sin(z) * zi;
        r[1] = (sin(z) - z * cos(z)) * zi * zi;
        for (int m = 2; m <= 16; ++m) r[m] = (2 * m - 1) * r[m - 1] * zi - r[m - 2];
        double zm = 1.0;
        for (int m = 0; m <= lmax; ++m) { j[m] = r[m] * zm; zm *= zi; }
    }
    for (int m = 0; m <= lmax; ++m)
        if (fabs(j[m]) < 1e-16) j[m] = 0.0;
}

/* Contracted Cartesian block (ab|cd), unnormalised components, row-major
 * [ncart(la)][ncart(lb)][ncart(lc)][ncart(ld)]. */
static void eri_cart(const or_shell *sa, const or_shell *sb, const or_shell *sc, const or_shell *sd, double *out)
{
    int la = sa->l, lb = sb->l, lc = sc->l, ld = sd->l;
    int Lab = la + lb, Lcd = lc + ld, L = Lab + Lcd;
    int NE = cart_offset(Lab + 1), NF = cart_offset(Lcd + 1);
    const double *A = sa->center, *B = sb->center, *C = sc->center, *D = sd->center;
    double AB2 = 0.0, CD2 = 0.0;
    for (int i = 0; i < 3; ++i) { AB2 += (A[i] - B[i]) * (A[i] - B[i]); CD2 += (C[i] - D[i]) * (C[i] - D[i]); }
    static __thread double V[NE_MAX][NE_MAX][OR_MAXLT + 1];
    static __thread double acc[NE_MAX][NE_MAX];
    memset(acc, 0, sizeof(acc));
    static __thread int comp[NE_MAX][3];
    for (int l = 0; l <= 4; ++l) {
        int cc[15][3]; list_cart(l, cc);
        for (int k = 0; k < ncart(l); ++k) memcpy(comp[cart_offset(l) + k], cc[k], sizeof(int) * 3);
    }
    for (int pa = 0; pa < sa->nprim; ++pa)
    for (int pb = 0; pb < sb->nprim; ++pb) {
        double a = sa->exps[pa], b = sb->exps[pb], zeta = a + b, sP = 1.0 / zeta;
        double UP = pow(M_PI * sP, 1.5) * exp(-a * b * sP * AB2);
        double P[3];
        for (int i = 0; i < 3; ++i) P[i] = (a * A[i] + b * B[i]) * sP;
        double ccab = scaled_cc(sa, pa) * scaled_cc(sb, pb);
        for (int pc = 0; pc < sc->nprim; ++pc)
        for (int pd = 0; pd < sd->nprim; ++pd) {
            double c = sc->exps[pc], d = sd->exps[pd], eta = c + d, sQ = 1.0 / eta;
            double UQ = pow(M_PI * sQ, 1.5) * exp(-c * d * sQ * CD2);
            double Q[3], W[3], PA[3], WP[3], QC[3], WQ[3], PQ2 = 0.0;
            double rho = zeta * eta / (zeta + eta);
            for (int i = 0; i < 3; ++i) {
                Q[i] = (c * C[i] + d * D[i]) * sQ;
                W[i] = (zeta * P[i] + eta * Q[i]) / (zeta + eta);
                PA[i] = P[i] - A[i]; WP[i] = W[i] - P[i];
                QC[i] = Q[i] - C[i]; WQ[i] = W[i] - Q[i];
                PQ2 += (P[i] - Q[i]) * (P[i] - Q[i]);
            }
            double F[OR_MAXLT + 1];
            if (g_op == 0) {
                oracle_boys(L, rho * PQ2, F);
                /* [00|00]^(m) = 2 pi^{5/2}/(zeta eta sqrt(zeta+eta)) K_AB K_CD F_m
                 *             = sqrt(2/pi) U_P U_Q sqrt(2 rho) F_m   (two_electron_fundamentals.c:71 at m=0) */
                double pre = sqrt(2.0 / M_PI) * UP * UQ * sqrt(2.0 * rho);
                for (int m = 0; m <= L; ++m) V[0][0][m] = pre * F[m];
            } else {
                /* j0(S r12): (-d/dT)^m of U_P U_Q exp(-S^2/(4 rho)) j0(S R), T = rho R^2 */
                double S = g_S, U = UP * UQ;
                if (S < 1e-14) {
                    V[0][0][0] = U;
                    for (int m = 1; m <= L; ++m) V[0][0][m] = 0.0;
                } else {
                    double eS = exp(-0.25 * S * S / rho), step = S * S / (2.0 * rho), sp = 1.0;
                    if (PQ2 < 1e-14) {
                        double df = 1.0;
                        for (int m = 0; m <= L; ++m) {
                            df *= (double)(2 * m + 1);
                            V[0][0][m] = U * eS * sp / df;
                            sp *= step;
                        }
                    } else {
                        oracle_sph_bessel(L, S * sqrt(PQ2), F);
                        for (int m = 0; m <= L; ++m) { V[0][0][m] = U * eS * sp * F[m]; sp *= step; }
                    }
                }
            }
            double o2z = 0.5 / zeta, o2e = 0.5 / eta, o2ze = 0.5 / (zeta + eta);
            double rz = rho / zeta, re = rho / eta;
            /* bra VRR */
            for (int g = 1; g < NE; ++g) {
                const int *e = comp[g];
                int le = e[0] + e[1] + e[2];
                int i = e[0] ? 0 : (e[1] ? 1 : 2);
                int em[3] = {e[0], e[1], e[2]}; em[i]--;
                int g1 = gidx(em[0], em[1], em[2]), g2 = -1;
                if (em[i] > 0) { int emm[3] = {em[0], em[1], em[2]}; emm[i]--; g2 = gidx(emm[0], emm[1], emm[2]); }
                for (int m = 0; m <= L - le; ++m) {
                    double v = PA[i] * V[g1][0][m] + WP[i] * V[g1][0][m + 1];
                    if (g2 >= 0) v += em[i] * o2z * (V[g2][0][m] - rz * V[g2][0][m + 1]);
                    V[g][0][m] = v;
                }
            }
            /* ket VRR */
            for (int h = 1; h < NF; ++h) {
                const int *f = comp[h];
                int lf = f[0] + f[1] + f[2];
                int i = f[0] ? 0 : (f[1] ? 1 : 2);
                int fm[3] = {f[0], f[1], f[2]}; fm[i]--;
                int h1 = gidx(fm[0], fm[1], fm[2]), h2 = -1;
                if (fm[i] > 0) { int fmm[3] = {fm[0], fm[1], fm[2]}; fmm[i]--; h2 = gidx(fmm[0], fmm[1], fmm[2]); }
                for (int g = 0; g < NE; ++g) {
                    const int *e = comp[g];
                    int le = e[0] + e[1] + e[2];
                    int g1 = -1;
                    if (e[i] > 0) { int em[3] = {e[0], e[1], e[2]}; em[i]--; g1 = gidx(em[0], em[1], em[2]); }
                    for (int m = 0; m <= L - le - lf; ++m) {
                        double v = QC[i] * V[g][h1][m] + WQ[i] * V[g][h1][m + 1];
                        if (h2 >= 0) v += fm[i] * o2e * (V[g][h2][m] - re * V[g][h2][m + 1]);
                        if (g1 >= 0) v += e[i] * o2ze * V[g1][h1][m + 1];
                        V[g][h][m] = v;
                    }
                }
            }
            double w = ccab * scaled_cc(sc, pc) * scaled_cc(sd, pd);
            for (int g = cart_offset(la); g < NE; ++g)
                for (int h = cart_offset(lc); h < NF; ++h) acc[g][h] += w * V[g][h][0];
        }
    }
    /* bra HRR: (a,b+1i| = (a+1i,b| + AB_i (a,b|  on contracted integrals, all ket f */
    static __thread double H1[NE_MAX][15][NE_MAX]; /* [a global][b cart idx within lb-level][f] */
    /* store by (a global, b global) using a small map: b global index <= cart_offset(lb+1) */
    static __thread double HB[NE_MAX][10][NE_MAX];
    int nbg = cart_offset(lb + 1);
    for (int g = 0; g < NE; ++g) for (int h = 0; h < NF; ++h) HB[g][0][h] = acc[g][h];
    double AB[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    double CD[3] = {C[0] - D[0], C[1] - D[1], C[2] - D[2]};
    for (int gb = 1; gb < nbg; ++gb) {
        const int *bb = comp[gb];
        int lbb = bb[0] + bb[1] + bb[2];
        int i = bb[0] ? 0 : (bb[1] ? 1 : 2);
        int bm[3] = {bb[0], bb[1], bb[2]}; bm[i]--;
        int gb1 = gidx(bm[0], bm[1], bm[2]);
        for (int ga = cart_offset(la); ga < cart_offset(Lab - lbb + 1); ++ga) {
            const int *aa = comp[ga];
            int ap[3] = {aa[0], aa[1], aa[2]}; ap[i]++;
            int gap = gidx(ap[0], ap[1], ap[2]);
            for (int h = cart_offset(lc); h < NF; ++h)
                HB[ga][gb][h] = HB[gap][gb1][h] + AB[i] * HB[ga][gb1][h];
        }
    }
    (void)H1;
    /* ket HRR on the (la, lb) bra block */
    int nca = ncart(la), ncb = ncart(lb), ncc = ncart(lc), ncd = ncart(ld);
    int ndg = cart_offset(ld + 1);
    static __thread double HK[15 * 15][NE_MAX][10];
    for (int ka = 0; ka < nca; ++ka)
        for (int kb = 0; kb < ncb; ++kb) {
            int ga = cart_offset(la) + ka, gb = cart_offset(lb) + kb, r = ka * ncb + kb;
            for (int h = 0; h < NF; ++h) HK[r][h][0] = (h >= cart_offset(lc)) ? HB[ga][gb][h] : 0.0;
            for (int gd = 1; gd < ndg; ++gd) {
                const int *dd = comp[gd];
                int ldd = dd[0] + dd[1] + dd[2];
                int i = dd[0] ? 0 : (dd[1] ? 1 : 2);
                int dm[3] = {dd[0], dd[1], dd[2]}; dm[i]--;
                int gd1 = gidx(dm[0], dm[1], dm[2]);
                for (int gc = cart_offset(lc); gc < cart_offset(Lcd - ldd + 1); ++gc) {
                    const int *cc = comp[gc];
                    int cp[3] = {cc[0], cc[1], cc[2]}; cp[i]++;
                    int gcp = gidx(cp[0], cp[1], cp[2]);
                    HK[r][gc][gd] = HK[r][gcp][gd1] + CD[i] * HK[r][gc][gd1];
                }
            }
            for (int kc = 0; kc < ncc; ++kc)
                for (int kd = 0; kd < ncd; ++kd)
                    out[((ka * ncb + kb) * ncc + kc) * ncd + kd] = HK[r][cart_offset(lc) + kc][cart_offset(ld) + kd];
        }
}

/* Spherical, normalised (ab|cd) block [(2la+1)][(2lb+1)][(2lc+1)][(2ld+1)]. */
int oracle_eri_quartet(const or_shell *sa, const or_shell *sb, const or_shell *sc, const or_shell *sd, double *out)
{
    if (sa->l > OR_MAXL || sb->l > OR_MAXL || sc->l > OR_MAXL || sd->l > OR_MAXL) return -1;
    double cart[1296];
    eri_cart(sa, sb, sc, sd, cart);
    int ls[4] = {sa->l, sb->l, sc->l, sd->l};
    to_spherical(4, ls, cart, out);
    return 0;
}

/* Whole-list helper for baselines: computes nq quartets given shell indices (4 per
 * quartet) into a scratch block and returns the sum of all values (so the work
 * cannot be optimised away). */
double oracle_eri_list(const or_shell *shells, int nq, const int *quads)
{
    double blk[1296], s = 0.0;
    for (int q = 0; q < nq; ++q) {
        const int *x = quads + 4 * q;
        oracle_eri_quartet(&shells[x[0]], &shells[x[1]], &shells[x[2]], &shells[x[3]], blk);
        int n = (2 * shells[x[0]].l + 1) * (2 * shells[x[1]].l + 1) * (2 * shells[x[2]].l + 1) * (2 * shells[x[3]].l + 1);
        for (int k = 0; k < n; ++k) s += blk[k];
    }
    return s;
}

int oracle_sizeof_shell(void) { return (int)sizeof(or_shell); }

/* ----------------------------------------------------------------------------------
 * Packed store: the screened unique shell quartets of a molecule and their blocks,
 * for systems whose dense N^4 tensor does not fit in host memory (upstream keeps the
 * dense tensor, Methods/hartree_fock.py:241-325 into Util/structures.py:506).  Each
 * quartet (a b | c d) lists shells a <= b, c <= d, with the pair (c, d) not after
 * (a, b) in pair order; its block is the spherical [na][nb][nc][nd] of
 * oracle_eri_quartet at offset boff[q].  Threads take quartets (or occupied orbitals)
 * in turn; nothing is shared between them but read-only inputs.
 * ---------------------------------------------------------------------------------- */
#include <pthread.h>

typedef struct {
    const or_shell *sh;
    const int *quads;
    const long long *boff;
    double *blocks;
    int nq, t, nt;
} or_eri_job;

static void *or_eri_worker(void *arg)
{
    or_eri_job *j = (or_eri_job *)arg;
    for (int q = j->t; q < j->nq; q += j->nt) {
        const int *x = j->quads + 4 * q;
        oracle_eri_quartet(&j->sh[x[0]], &j->sh[x[1]], &j->sh[x[2]], &j->sh[x[3]], j->blocks + j->boff[q]);
    }
    return NULL;
}

/* Blocks of nq quartets into blocks[boff[q] ...], on nthreads threads. */
int oracle_eri_blocks(const or_shell *shells, int nq, const int *quads, const long long *boff, double *blocks,
                      int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    or_eri_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (or_eri_job){shells, quads, boff, blocks, nq, t, nthreads};
        if (pthread_create(&th[t], NULL, or_eri_worker, &jobs[t]) != 0) return -1;
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* The distinct index permutations (p q | r s) of one unique element: the 8 images of
 * the permutational symmetry with repeats removed.  Returns their count. */
static int or_images(int m, int n, int l, int s, int img[8][4])
{
    const int cand[8][4] = {{m, n, l, s}, {n, m, l, s}, {m, n, s, l}, {n, m, s, l},
                            {l, s, m, n}, {s, l, m, n}, {l, s, n, m}, {s, l, n, m}};
    int k = 0;
    for (int c = 0; c < 8; ++c) {
        int dup = 0;
        for (int e = 0; e < k && !dup; ++e)
            dup = img[e][0] == cand[c][0] && img[e][1] == cand[c][1] && img[e][2] == cand[c][2] &&
                  img[e][3] == cand[c][3];
        if (!dup) {
            for (int i = 0; i < 4; ++i) img[k][i] = cand[c][i];
            ++k;
        }
    }
    return k;
}

/* Visit every unique element of quartet q once: within a block whose two shells of a
 * pair coincide only one of (mu nu) / (nu mu) is unique, and for a quartet whose bra
 * and ket pairs coincide only one of (mu nu | lam sig) / (lam sig | mu nu). */
#define OR_FOR_UNIQUE(sh, ao, x, blk, ...)                                                               \
    do {                                                                                                 \
        const int a_ = (x)[0], b_ = (x)[1], c_ = (x)[2], d_ = (x)[3];                                    \
        const int na_ = 2 * (sh)[a_].l + 1, nb_ = 2 * (sh)[b_].l + 1, nc_ = 2 * (sh)[c_].l + 1,          \
                  nd_ = 2 * (sh)[d_].l + 1;                                                              \
        const int same_bra_ket_ = a_ == c_ && b_ == d_;                                                  \
        for (int i_ = 0; i_ < na_; ++i_)                                                                 \
            for (int j_ = 0; j_ < nb_; ++j_) {                                                           \
                if (a_ == b_ && j_ > i_) continue;                                                       \
                for (int k_ = 0; k_ < nc_; ++k_)                                                         \
                    for (int l_ = 0; l_ < nd_; ++l_) {                                                   \
                        if (c_ == d_ && l_ > k_) continue;                                               \
                        if (same_bra_ket_ && (k_ * nd_ + l_) > (i_ * nb_ + j_)) continue;                \
                        const double v = (blk)[((i_ * nb_ + j_) * nc_ + k_) * nd_ + l_];                 \
                        const int mu = (ao)[a_] + i_, nu = (ao)[b_] + j_, la = (ao)[c_] + k_,            \
                                  si = (ao)[d_] + l_;                                                    \
                        __VA_ARGS__                                                                      \
                    }                                                                                    \
            }                                                                                            \
    } while (0)

typedef struct {
    const or_shell *sh;
    const int *ao, *quads;
    const long long *boff;
    const double *blocks, *Dj, *Dk;
    double *J, *K;
    int nq, n, t, nt;
} or_jk_job;

static void *or_jk_worker(void *arg)
{
    or_jk_job *j = (or_jk_job *)arg;
    const int n = j->n;
    for (int q = j->t; q < j->nq; q += j->nt) {
        const int *x = j->quads + 4 * q;
        const double *blk = j->blocks + j->boff[q];
        OR_FOR_UNIQUE(j->sh, j->ao, x, blk, {
            int img[8][4];
            const int ni = or_images(mu, nu, la, si, img);
            for (int e = 0; e < ni; ++e) {
                const int p = img[e][0], qq = img[e][1], r = img[e][2], s = img[e][3];
                j->J[p * n + qq] += j->Dj[r * n + s] * v;  /* J_pq = sum_rs (pq|rs) Dj_rs */
                j->K[p * n + s] += j->Dk[r * n + qq] * v;  /* K_ps = sum_qr (pq|rs) Dk_rq */
            }
        });
    }
    return NULL;
}

/* J = einsum('cd,abcd->ab', Dj, ERI) and K = einsum('cb,abcd->ad', Dk, ERI) over the
 * packed store (Methods/hartree_fock.py:345-347); ao[shell] = first AO of the shell,
 * J and K (n x n) are overwritten. */
int oracle_jk_packed(const or_shell *shells, const int *ao, int nq, const int *quads, const long long *boff,
                     const double *blocks, int n, const double *Dj, const double *Dk, double *J, double *K,
                     int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    const size_t nn = (size_t)n * n;
    double *buf = (double *)calloc((size_t)nthreads * 2 * nn, sizeof(double));
    if (!buf) return -1;
    pthread_t th[256];
    or_jk_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (or_jk_job){shells, ao, quads, boff, blocks, Dj, Dk, buf + 2 * t * nn, buf + (2 * t + 1) * nn,
                              nq, n, t, nthreads};
        if (pthread_create(&th[t], NULL, or_jk_worker, &jobs[t]) != 0) { free(buf); return -1; }
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    for (size_t e = 0; e < nn; ++e) {
        double sj = 0.0, sk = 0.0;
        for (int t = 0; t < nthreads; ++t) { sj += buf[2 * t * nn + e]; sk += buf[(2 * t + 1) * nn + e]; }
        J[e] = sj;
        K[e] = sk;
    }
    free(buf);
    return 0;
}

typedef struct {
    const or_shell *sh;
    const int *ao, *quads;
    const long long *boff;
    const double *blocks, *C;
    double *T;
    int nq, n, o, i0, i1;
} or_q1_job;

static void *or_q1_worker(void *arg)
{
    or_q1_job *j = (or_q1_job *)arg;
    const int n = j->n, o = j->o;
    const long long np = (long long)n * (n + 1) / 2;
    for (int q = 0; q < j->nq; ++q) {
        const int *x = j->quads + 4 * q;
        const double *blk = j->blocks + j->boff[q];
        OR_FOR_UNIQUE(j->sh, j->ao, x, blk, {
            int img[8][4];
            const int ni = or_images(mu, nu, la, si, img);
            for (int e = 0; e < ni; ++e) {
                const int p = img[e][0], qq = img[e][1], r = img[e][2], s = img[e][3];
                if (r < s) continue;  /* the (s r) image carries the same pair */
                const long long rs = (long long)r * (r + 1) / 2 + s;
                for (int i = j->i0; i < j->i1; ++i)
                    j->T[((long long)i * n + qq) * np + rs] += j->C[(long long)p * o + i] * v;
            }
        });
    }
    return NULL;
}

/* First quarter of the MP2 AO->MO transform (Methods/mp2.py:43-69) over the packed
 * store: T[i][nu][rs] = sum_mu C[mu][i] (mu nu | r s) for the o columns of C (n x o,
 * row-major) and the lower-triangle pair index rs = r(r+1)/2 + s, r >= s.  T
 * (o x n x n(n+1)/2) is accumulated into (zero it first).  Threads split the
 * occupied index, so each reads the whole store. */
int oracle_mp2_first_quarter(const or_shell *shells, const int *ao, int nq, const int *quads,
                             const long long *boff, const double *blocks, int n, int o, const double *C, double *T,
                             int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > o) nthreads = o;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    or_q1_job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        const int i0 = (int)((long long)o * t / nthreads), i1 = (int)((long long)o * (t + 1) / nthreads);
        jobs[t] = (or_q1_job){shells, ao, quads, boff, blocks, C, T, nq, n, o, i0, i1};
        if (pthread_create(&th[t], NULL, or_q1_worker, &jobs[t]) != 0) return -1;
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

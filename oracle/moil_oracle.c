/*
 * moil_oracle.c -- CPU FP64 restatement of MOIL's nonbonded Ewald path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): nothing in the product links, loads
 * or calls this file.  It exists so the GPU library can be checked against
 * MOIL's own algorithm on the same inputs, and so the CPU baseline can be
 * timed.  Citations are MOIL source files (paths relative to the MOIL tree).
 *
 * Parity status: MOIL itself cannot be compiled here (no Fortran compiler),
 * and MOIL ships no test vectors.  The restatement is pinned by physics
 * known-answer tests (NaCl Madelung constant, two-charge Ewald sum), by
 * central finite differences of its own energy, and by the agreement of the
 * MOIL list path (13 image translations) with an independent minimum-image
 * evaluator.
 */
#include "moil_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KOFDIE 332.0716            /* COMMON/CONVERT.BLOCK:13 */
#define PERFT 10000                 /* COMMON/LENGTH_SAVE_PRESS.BLOCK:231 */
#define PI_D 3.14159265358979323846

/* ------------------------------------------------------------------------ */
/* erfc, Ewald coefficient, spline table                                     */

/* symm/ewald_init.f:298-335: doubling search then 60+i bisection steps on
 * erfc(x*rc)/rc >= dtol.  libm erfc stands in for CALERF (symm/erfcfun.f). */
double ora_find_ewaldcof(double cutoff, double dtol)
{
    double x = 0.5, xlo, xhi, term;
    int i = 0, n;
    do {
        x = 2.0 * x;
        i++;
        term = erfc(x * cutoff) / cutoff;
    } while (term >= dtol);
    n = i + 60;
    xlo = 0.0;
    xhi = x;
    for (i = 1; i <= n; i++) {
        x = (xlo + xhi) / 2;
        term = erfc(x * cutoff) / cutoff;
        if (term >= dtol) xlo = x; else xhi = x;
    }
    return x;
}

/* de Boor cubspl (symm/ewald_init.f:453-574) for slope boundary conditions at
 * both ends (ibcbeg = ibcend = 1), the only case MOIL uses.  c is c(4,n),
 * column-major, 1-based in the comments.  On entry c(1,i) are the values and
 * c(2,1), c(2,n) the end slopes; on exit c(1..4,i) are the Taylor
 * coefficients of the piece on [tau(i), tau(i+1)]. */
static void cubspl_slope(const double *tau, double *c, int n)
{
#define C(j, i) c[4 * ((i) - 1) + ((j) - 1)]
#define T(i) tau[(i) - 1]
    int l = n - 1, m, i, j;
    double g, dtau, divdf1, divdf3;
    for (m = 2; m <= n; m++) {
        C(3, m) = T(m) - T(m - 1);
        C(4, m) = (C(1, m) - C(1, m - 1)) / C(3, m);
    }
    C(4, 1) = 1.0;
    C(3, 1) = 0.0;
    if (n > 2) {
        for (m = 2; m <= l; m++) {
            g = -C(3, m + 1) / C(4, m - 1);
            C(2, m) = g * C(2, m - 1) + 3.0 * (C(3, m) * C(4, m + 1) + C(3, m + 1) * C(4, m));
            C(4, m) = g * C(3, m - 1) + 2.0 * (C(3, m) + C(3, m + 1));
        }
    }
    /* slope prescribed at the right end: straight to back substitution */
    for (j = l; j >= 1; j--)
        C(2, j) = (C(2, j) - C(3, j) * C(2, j + 1)) / C(4, j);
    for (i = 2; i <= n; i++) {
        dtau = C(3, i);
        divdf1 = (C(1, i) - C(1, i - 1)) / dtau;
        divdf3 = C(2, i - 1) + C(2, i) - 2.0 * divdf1;
        C(3, i - 1) = 2.0 * (divdf1 - C(2, i - 1) - divdf3) / dtau;
        C(4, i - 1) = (divdf3 / dtau) * (6.0 / dtau);
    }
#undef C
#undef T
}

/* symm/ewald_init.f:101-126 + fill_erf_table (:418-449): erftbdns = perft/2
 * points per unit of alpha*r, up to 1.5*cutoff. */
int ora_erfc_table(double ewaldcof, double cutoff, double *tab, int cap)
{
    double erftbdns = 0.5 * PERFT;
    double del = 1.0 / erftbdns;
    double fac = 2.0 / sqrt(PI_D);
    int mx = (int)(ewaldcof * erftbdns * cutoff * 1.5), i;
    double *tau;
    if (mx > cap || mx < 3) return -mx;
    tau = (double *)malloc(sizeof(double) * mx);
    memset(tab, 0, sizeof(double) * 4 * mx);
    tab[1] = -fac;                                    /* erf_arr(2,1) */
    {
        double x = (mx - 1) * del;
        tab[4 * (mx - 1) + 1] = -fac * exp(-x * x);   /* erf_arr(2,mx) */
    }
    for (i = 1; i <= mx; i++) {
        double x = del * (i - 1);
        tau[i - 1] = x;
        tab[4 * (i - 1)] = erfc(x);
    }
    cubspl_slope(tau, tab, mx);
    free(tau);
    return mx;
}

/* The lookup every MOIL Ewald kernel inlines (e.g. pot/cdie_ewald.f:148-160):
 * erfcc = c1 + dx*(c2 + dx/2*(c3 + dx*c4/3)), derfc = -(c2 + dx*(c3 + dx*c4/2)). */
double ora_erfc_table_eval(const double *tab, double erftbdns, double x, double *derfc)
{
    int ind = (int)(erftbdns * x) + 1;
    double del = 1.0 / erftbdns;
    double dx = x - (ind - 1) * del;
    const double *e = tab + 4 * (ind - 1);
    *derfc = -e[1] - dx * (e[2] + 0.5 * dx * e[3]);
    return dx * (e[1] + 0.5 * dx * (e[2] + dx * e[3] * (1.0 / 3.0))) + e[0];
}

/* ------------------------------------------------------------------------ */
/* common evaluation context                                                  */

typedef struct ctx {
    const ora_input *in;
    int npt;
    double cutvdw2, cutvbig2, cutele2, cutebig2, cutmono2;
    double ewaldcof, epstmp;
    double *tab;
    int ntab;
    double erftbdns;
    double *coor;       /* working copy (squeezed) */
    char *flagchr;
    char *iswat;        /* per monomer */
    int *first;         /* first atom (1-based) of each monomer */
    double ron2, roff2, swden;
} ctx;

static void erfc_pair(const ctx *c, double x, double *erfcc, double *derfc)
{
    if (c->in->erfc_mode == 0) {
        *erfcc = ora_erfc_table_eval(c->tab, c->erftbdns, x, derfc);
    } else {
        *erfcc = erfc(x);
        *derfc = 2.0 / sqrt(PI_D) * exp(-x * x);
    }
}

/* LJ switch extension (off in MOIL parity): scales e1 and adjusts df1 = dE/dr / r. */
static void lj_switch(const ctx *c, double r2, double *e1, double *df1)
{
    if (!c->in->lj_switch || r2 <= c->ron2) return;
    {
        double u = r2, d = c->roff2 - u;
        double sw = d * d * (c->roff2 + 2.0 * u - 3.0 * c->ron2) * c->swden;
        double dsw = 12.0 * d * (c->ron2 - u) * c->swden;   /* (dsw/dr)/r */
        *df1 = *df1 * sw + *e1 * dsw;
        *e1 *= sw;
    }
}

static int ctx_init(ctx *c, const ora_input *in)
{
    int i, m;
    double rvbg, rebg;
    memset(c, 0, sizeof(*c));
    c->in = in;
    c->npt = in->npt;
    rvbg = in->rvbg >= 0 ? in->rvbg : in->rvmx + 2.0;      /* pot/energy.f:388-389 */
    rebg = in->rebg >= 0 ? in->rebg : in->relx + 2.0;
    c->cutvdw2 = in->rvmx * in->rvmx;
    c->cutvbig2 = rvbg * rvbg;
    c->cutele2 = in->relx * in->relx;
    c->cutebig2 = rebg * rebg;
    c->cutmono2 = in->cutm > 0 ? in->cutm * in->cutm : c->cutebig2 * 1.44;   /* :396-399 */
    c->ewaldcof = in->ewaldcof > 0 ? in->ewaldcof : ora_find_ewaldcof(in->relx, in->dtol);
    c->epstmp = KOFDIE / in->eps;
    c->erftbdns = 0.5 * PERFT;
    c->ntab = (int)(c->ewaldcof * c->erftbdns * in->relx * 1.5);
    c->tab = (double *)malloc(sizeof(double) * 4 * (c->ntab + 8));
    if (ora_erfc_table(c->ewaldcof, in->relx, c->tab, c->ntab + 8) <= 0) return -1;
    c->coor = (double *)malloc(sizeof(double) * 3 * in->npt);
    memcpy(c->coor, in->coor, sizeof(double) * 3 * in->npt);
    c->flagchr = (char *)malloc(in->npt);
    for (i = 0; i < in->npt; i++) c->flagchr[i] = fabs(in->ptchg[i]) > 1e-6;  /* connect/chsort.f:17-24 */
    c->iswat = (char *)malloc(in->totmon + 1);
    c->first = (int *)malloc(sizeof(int) * (in->totmon + 1));
    for (m = 0; m < in->totmon; m++) {
        c->iswat[m] = in->montype[m] == 1;
        c->first[m] = m == 0 ? 1 : in->poipt[m - 1] + 1;
    }
    c->ron2 = in->r_on * in->r_on;
    c->roff2 = c->cutvdw2;
    if (in->lj_switch) {
        double d = c->roff2 - c->ron2;
        c->swden = 1.0 / (d * d * d);
    }
    return 0;
}

static void ctx_free(ctx *c)
{
    free(c->tab); free(c->coor); free(c->flagchr); free(c->iswat); free(c->first);
}

#define X(i) c->coor[3 * ((i) - 1)]
#define Y(i) c->coor[3 * ((i) - 1) + 1]
#define Z(i) c->coor[3 * ((i) - 1) + 2]
#define DP(k, i) dpot[3 * ((i) - 1) + (k)]

/* symm/squeeze.f:66-145: water and ion monomers are moved back by one box
 * length when their first atom is outside [-L/2, L/2] (y, x, z order). */
static void squeeze(ctx *c)
{
    const ora_input *in = c->in;
    int m, k;
    double ha = in->a * 0.5, hb = in->b * 0.5, hc = in->c * 0.5;
    for (m = 0; m < in->totmon; m++) {
        int is = c->first[m], ie = in->poipt[m];
        double xc, yc, zc;
        if (in->montype[m] == 0) continue;
        xc = X(is); yc = Y(is); zc = Z(is);
        if (yc < -hb) for (k = is; k <= ie; k++) Y(k) += in->b;
        if (yc > hb) for (k = is; k <= ie; k++) Y(k) -= in->b;
        if (xc < -ha) for (k = is; k <= ie; k++) X(k) += in->a;
        if (zc < -hc) for (k = is; k <= ie; k++) Z(k) += in->c;
        if (xc > ha) for (k = is; k <= ie; k++) X(k) -= in->a;
        if (zc > hc) for (k = is; k <= ie; k++) Z(k) -= in->c;
    }
}

/* ------------------------------------------------------------------------ */
/* lists (pot/nbondm.f, pot/nbond.f, symm/syminit.f, symm/nbmsym.f, nbsym.f) */

typedef struct ivec { int *v; long long n, cap; } ivec;
static void ipush(ivec *a, int x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 1024;
        a->v = (int *)realloc(a->v, sizeof(int) * a->cap);
    }
    a->v[a->n++] = x;
}

typedef struct lists {
    /* primary atom lists, CSR by atom: point[0..npt] (point[l] = end after atom l) */
    int *point1, *point2, *point3;
    ivec list1, list2, list3;
    /* primary water lists, by water ordinal 1..nwaters */
    int nwaters;
    int *indxwat;            /* water ordinal -> monomer (0-based) */
    int *poinwat1, *poinwat2;/* 0..nwaters */
    ivec listwt1, listwt2;   /* monomer numbers (0-based) */
    /* image lists, per translation: (real atom, end pointer) blocks */
    int symop[13][3];
    ivec symreal1, symreal2, symreal3, psym1, psym2, psym3;
    int iblock1[14], iblock2[14], iblock3[14];
    ivec symmwat1, symmwat2, psymwt1, psymwt2;
    int iblckwt1[14], iblckwt2[14];
    long long nprim1, nprim2, nprim3, nprimw1, nprimw2;
} lists;

static int excluded(const ora_input *in, int l, int m)
{
    int k;
    for (k = in->exc1[l - 1] + 1; k <= in->exc1[l]; k++)
        if (in->exc2[k - 1] == m) return 1;
    return 0;
}

/* nbond.f:115-149 / nbsym.f:92-137: hydrogen rule then list1/list2/list3 */
static void classify(const ctx *c, lists *L, int l, int m, double r2, int *n1, int *n2, int *n3)
{
    const ora_input *in = c->in;
    /* nbsym applies the hydrogen rule unconditionally, nbond only under hvdw0 */
    {
        int flag2 = (!in->arith) && (r2 < c->cutebig2) &&
                    (in->epsgm12[l - 1] < 1e-3 || in->epsgm12[m - 1] < 1e-3);
        if (flag2 && c->flagchr[l - 1] && c->flagchr[m - 1]) {
            ipush(&L->list3, m); (*n3)++;
            return;
        } else if (flag2) {
            return;
        }
    }
    if (r2 < c->cutvbig2) {
        if (c->flagchr[l - 1] && c->flagchr[m - 1]) { ipush(&L->list1, m); (*n1)++; }
        else { ipush(&L->list2, m); (*n2)++; }
    } else if (r2 < c->cutebig2) {
        if (c->flagchr[l - 1] && c->flagchr[m - 1]) { ipush(&L->list3, m); (*n3)++; }
    }
}

static void build_lists(const ctx *c, lists *L)
{
    const ora_input *in = c->in;
    int M = in->totmon, npt = in->npt;
    double *cent = (double *)malloc(sizeof(double) * 3 * M);
    int *pointm = (int *)malloc(sizeof(int) * (M + 2));
    ivec nblistm = {0};
    int i, j, l, m, nlist = 0, iwat = 0, nflag = 0;
    int nwl1 = 0, nwl2 = 0;
    memset(L, 0, sizeof(*L));

    /* nbondm.f:79-124: centroids (water: its oxygen) */
    for (i = 0; i < M; i++) {
        int is = c->first[i], ie = in->poipt[i];
        if (c->iswat[i]) {
            int o = ie - 2;
            cent[3 * i] = X(o); cent[3 * i + 1] = Y(o); cent[3 * i + 2] = Z(o);
        } else {
            double sx = 0, sy = 0, sz = 0, r;
            for (j = is; j <= ie; j++) { sx += X(j); sy += Y(j); sz += Z(j); }
            r = 1.0 / (double)(ie - is + 1);
            cent[3 * i] = sx * r; cent[3 * i + 1] = sy * r; cent[3 * i + 2] = sz * r;
        }
    }
    L->nwaters = 0;
    for (i = 0; i < M; i++) L->nwaters += c->iswat[i];
    L->indxwat = (int *)malloc(sizeof(int) * (L->nwaters + 2));
    L->poinwat1 = (int *)calloc(L->nwaters + 2, sizeof(int));
    L->poinwat2 = (int *)calloc(L->nwaters + 2, sizeof(int));

    /* nbondm.f:143-218: O(M^2) monomer pair loop */
    for (i = 0; i < M; i++) {
        int watflag = c->iswat[i];
        nlist++;
        pointm[i] = nlist;
        if (nblistm.n < nlist) ipush(&nblistm, i); else nblistm.v[nlist - 1] = i;
        if (watflag) {
            if (nflag) {
                nlist--;
                pointm[i] = nlist;
                nblistm.v[nlist - 1] = i;
                nblistm.n = nlist;
            }
            iwat++;
            L->indxwat[iwat] = i;
            L->poinwat1[iwat] = nwl1;
            L->poinwat2[iwat] = nwl2;
            nflag = 1;
        } else {
            nflag = 0;
        }
        if (i == M - 1) continue;
        for (j = i + 1; j < M; j++) {
            double rx, r2;
            rx = cent[3 * i] - cent[3 * j]; r2 = rx * rx;
            if (r2 > c->cutmono2) continue;
            rx = cent[3 * i + 1] - cent[3 * j + 1]; r2 += rx * rx;
            if (r2 > c->cutmono2) continue;
            rx = cent[3 * i + 2] - cent[3 * j + 2]; r2 += rx * rx;
            if (watflag && c->iswat[j]) {
                if (r2 <= c->cutvbig2) { ipush(&L->listwt1, j); nwl1++; }
                else if (r2 <= c->cutebig2) { ipush(&L->listwt2, j); nwl2++; }
            } else if (r2 <= c->cutmono2) {
                nlist++;
                if (nblistm.n < nlist) ipush(&nblistm, j); else nblistm.v[nlist - 1] = j;
                nblistm.n = nlist;
                nflag = 0;
            }
        }
    }
    pointm[M] = nflag ? nlist : nlist + 1;
    /* my_nwat = nwaters - 1 (nbondm.f:225): the end pointer of ordinal nwaters-1
     * is the start pointer stored when the last water was visited */
    L->poinwat1[L->nwaters + 1] = nwl1;
    L->poinwat2[L->nwaters + 1] = nwl2;

    /* nbond.f:54-157: atom lists over the monomer list */
    L->point1 = (int *)calloc(npt + 1, sizeof(int));
    L->point2 = (int *)calloc(npt + 1, sizeof(int));
    L->point3 = (int *)calloc(npt + 1, sizeof(int));
    {
        int n1 = 0, n2 = 0, n3 = 0;
        for (i = 0; i < M; i++) {
            int ki = c->first[i], jb = pointm[i], je = pointm[i + 1] - 1, jj;
            for (l = ki; l <= in->poipt[i]; l++) {
                for (jj = jb; jj <= je; jj++) {
                    int kmon = nblistm.v[jj - 1], kj;
                    kj = (kmon != i) ? c->first[kmon] : l + 1;
                    for (m = kj; m <= in->poipt[kmon]; m++) {
                        double rx, ry, rz, r2;
                        if (excluded(in, l, m)) continue;
                        rx = X(l) - X(m); ry = Y(l) - Y(m); rz = Z(l) - Z(m);
                        r2 = rx * rx + ry * ry + rz * rz;
                        if (in->hvdw0) classify(c, L, l, m, r2, &n1, &n2, &n3);
                        else {
                            if (r2 < c->cutvbig2) {
                                if (c->flagchr[l - 1] && c->flagchr[m - 1]) { ipush(&L->list1, m); n1++; }
                                else { ipush(&L->list2, m); n2++; }
                            } else if (r2 < c->cutebig2 && c->flagchr[l - 1] && c->flagchr[m - 1]) {
                                ipush(&L->list3, m); n3++;
                            }
                        }
                    }
                }
                L->point1[l] = n1; L->point2[l] = n2; L->point3[l] = n3;
            }
        }
        /* atoms never visited (none in practice) keep their predecessor's pointer */
        for (l = 1; l <= npt; l++) {
            if (L->point1[l] < L->point1[l - 1]) L->point1[l] = L->point1[l - 1];
            if (L->point2[l] < L->point2[l - 1]) L->point2[l] = L->point2[l - 1];
            if (L->point3[l] < L->point3[l - 1]) L->point3[l] = L->point3[l - 1];
        }
    }
    L->nprim1 = L->list1.n; L->nprim2 = L->list2.n; L->nprim3 = L->list3.n;
    L->nprimw1 = L->listwt1.n; L->nprimw2 = L->listwt2.n;

    /* syminit.f:80-164: the 13 half-shell translations, in MOIL's order */
    {
        static const int ops[13][3] = {
            {1, 0, 1}, {1, 0, 0}, {1, 0, -1}, {0, 0, 1}, {1, 1, 1}, {1, 1, 0}, {1, 1, -1},
            {0, 1, 1}, {0, 1, 0}, {0, 1, -1}, {1, -1, 1}, {1, -1, 0}, {1, -1, -1}};
        memcpy(L->symop, ops, sizeof(ops));
    }
    {
        double ha = 0.5 * in->a, hb = 0.5 * in->b, hc = 0.5 * in->c;
        double large = c->cutmono2;
        int *need = (int *)malloc(sizeof(int) * M);
        int *pm = (int *)malloc(sizeof(int) * (M + 1));
        ivec nbm = {0};
        int ipwat1 = 0, ipwat2 = 0, isym;
        int ind1 = 0, ind2 = 0, ind3 = 0;
        L->iblock1[0] = L->iblock2[0] = L->iblock3[0] = 0;
        L->iblckwt1[0] = L->iblckwt2[0] = 0;
        for (isym = 1; isym <= 13; isym++) {
            int ia = L->symop[isym - 1][0], jb = L->symop[isym - 1][1], kc = L->symop[isym - 1][2];
            double da = ia * in->a, db = jb * in->b, dc = kc * in->c;
            double barx = 0.5 * da, bary = 0.5 * db, barz = 0.5 * dc;
            int nneed = 0, nl = 0;
            large = c->cutmono2;
            /* nbmsym.f:80-89: any centroid outside the box widens the test */
            for (i = 0; i < M; i++)
                if (fabs(cent[3 * i]) > ha || fabs(cent[3 * i + 1]) > hb || fabs(cent[3 * i + 2]) > hc) {
                    large = c->cutmono2 * 4.0;
                    break;
                }
            /* nbmsym.f:92-112: real monomers near the translated face */
            for (i = 0; i < M; i++) {
                double cl;
                if (ia) { cl = cent[3 * i] - barx; if (cl * cl > c->cutmono2) continue; }
                if (jb) { cl = cent[3 * i + 1] - bary; if (cl * cl > c->cutmono2) continue; }
                if (kc) { cl = cent[3 * i + 2] - barz; if (cl * cl > c->cutmono2) continue; }
                need[nneed++] = i;
            }
            nbm.n = 0;
            /* nbmsym.f:161-246 */
            for (i = 0; i < M; i++) {
                double sx = cent[3 * i] + da, sy = cent[3 * i + 1] + db, sz = cent[3 * i + 2] + dc;
                double xch = fabs(sx) - ha, ych = fabs(sy) - hb, zch = fabs(sz) - hc;
                int watflag, oneig1 = 0, oneig2 = 0, kk;
                if (xch < 0) xch = 0;
                if (ych < 0) ych = 0;
                if (zch < 0) zch = 0;
                if (xch * xch + ych * ych + zch * zch > large) { pm[i] = nl; continue; }
                watflag = c->iswat[i];
                for (kk = 0; kk < nneed; kk++) {
                    double rx, r2;
                    j = need[kk];
                    rx = sx - cent[3 * j]; r2 = rx * rx;
                    if (r2 > c->cutmono2) continue;
                    rx = sy - cent[3 * j + 1]; r2 += rx * rx;
                    if (r2 > c->cutmono2) continue;
                    rx = sz - cent[3 * j + 2]; r2 += rx * rx;
                    if (watflag && c->iswat[j]) {
                        if (r2 < c->cutvbig2) { oneig1 = 1; ipush(&L->listwt1, j); }
                        else if (r2 < c->cutebig2) { oneig2 = 1; ipush(&L->listwt2, j); }
                    } else if (r2 < c->cutmono2) {
                        nl++;
                        ipush(&nbm, j);
                    }
                }
                pm[i] = nl;
                if (watflag) {
                    if (oneig1) { ipwat1++; ipush(&L->symmwat1, i); ipush(&L->psymwt1, 0); }
                    if (oneig2) { ipwat2++; ipush(&L->symmwat2, i); ipush(&L->psymwt2, 0); }
                    if (ipwat1) L->psymwt1.v[ipwat1 - 1] = (int)L->listwt1.n;
                    if (ipwat2) L->psymwt2.v[ipwat2 - 1] = (int)L->listwt2.n;
                }
            }
            L->iblckwt1[isym] = ipwat1;
            L->iblckwt2[isym] = ipwat2;
            /* nbsym.f:69-186: atom pairs between translated and real monomers */
            {
                int jbeg = 1, ki = 1, ii;
                for (ii = 0; ii < M; ii++) {
                    int jend = pm[ii];
                    for (l = ki; l <= in->poipt[ii]; l++) {
                        int n1 = 0, n2 = 0, n3 = 0, jj;
                        double xl = X(l) + da, yl = Y(l) + db, zl = Z(l) + dc;
                        for (jj = jbeg; jj <= jend; jj++) {
                            int kmon = nbm.v[jj - 1];
                            for (m = c->first[kmon]; m <= in->poipt[kmon]; m++) {
                                double rx = xl - X(m), ry = yl - Y(m), rz = zl - Z(m);
                                double r2 = rx * rx + ry * ry + rz * rz;
                                classify(c, L, l, m, r2, &n1, &n2, &n3);
                            }
                        }
                        if (n1) { ind1++; ipush(&L->symreal1, l); ipush(&L->psym1, 0); }
                        if (n2) { ind2++; ipush(&L->symreal2, l); ipush(&L->psym2, 0); }
                        if (n3) { ind3++; ipush(&L->symreal3, l); ipush(&L->psym3, 0); }
                        if (ind1) L->psym1.v[ind1 - 1] = (int)L->list1.n;
                        if (ind2) L->psym2.v[ind2 - 1] = (int)L->list2.n;
                        if (ind3) L->psym3.v[ind3 - 1] = (int)L->list3.n;
                    }
                    ki = in->poipt[ii] + 1;
                    jbeg = pm[ii] + 1;
                }
            }
            L->iblock1[isym] = ind1; L->iblock2[isym] = ind2; L->iblock3[isym] = ind3;
        }
        free(need); free(pm); free(nbm.v);
    }
    free(cent); free(pointm); free(nblistm.v);
}

static void free_lists(lists *L)
{
    free(L->point1); free(L->point2); free(L->point3);
    free(L->list1.v); free(L->list2.v); free(L->list3.v);
    free(L->indxwat); free(L->poinwat1); free(L->poinwat2);
    free(L->listwt1.v); free(L->listwt2.v);
    free(L->symreal1.v); free(L->symreal2.v); free(L->symreal3.v);
    free(L->psym1.v); free(L->psym2.v); free(L->psym3.v);
    free(L->symmwat1.v); free(L->symmwat2.v); free(L->psymwt1.v); free(L->psymwt2.v);
}

/* ------------------------------------------------------------------------ */
/* pair terms                                                                 */

/* LJ a, b for the pair as cdie_ewald.f:377-383 / 432-472 compute them */
static void lj_ab(const ctx *c, int i, int j, double s2, double *a, double *b)
{
    const ora_input *in = c->in;
    double s6 = s2 * s2 * s2;
    if (!in->arith) {
        *a = in->epsgm12[i - 1] * in->epsgm12[j - 1] * s6 * s6;
        *b = in->epsgm6[i - 1] * in->epsgm6[j - 1] * s6;
    } else {
        double aa = in->epsgm12[i - 1] * in->epsgm12[j - 1];
        double bb = 0.5 * (in->epsgm6[i - 1] + in->epsgm6[j - 1]);
        double b1 = bb * bb * bb;
        b1 = b1 * b1;
        *b = aa * b1 * s6;
        b1 = b1 * b1;
        *a = aa * b1 * s6 * s6;
    }
}

/* One atom pair of list1/list2/list3 (cdie_ewald.f:313-671, symcdie_ewald.f).
 * kind 1: LJ if r2 <= cutvdw2, Coulomb always; 2: LJ only (r2 <= cutvdw2);
 * 3: Coulomb if r2 <= cutele2.  xi are the (possibly translated) i coordinates. */
static void atom_pair(const ctx *c, int kind, int i, double xi, double yi, double zi, int j,
                      double *dpot, int addi, double *evdw, double *eel, double *vir, ora_output *out)
{
    const ora_input *in = c->in;
    double rx = xi - X(j), ry = yi - Y(j), rz = zi - Z(j);
    double r2 = rx * rx + ry * ry + rz * rz, s2, df1 = 0, df2 = 0, e1 = 0, e2 = 0, df;
    int lj = 0, el = 0;
    if (kind == 1) { lj = r2 <= c->cutvdw2; el = 1; }
    else if (kind == 2) { lj = r2 <= c->cutvdw2; }
    else { el = r2 <= c->cutele2; }
    if (!lj && !el) return;
    s2 = 1.0 / r2;
    if (lj) {
        double a, b;
        lj_ab(c, i, j, s2, &a, &b);
        e1 = a - b;
        df1 = -6.0 * s2 * (a + e1);
        lj_switch(c, r2, &e1, &df1);
        *evdw += e1;
        *vir -= df1 * r2;            /* cdie_ewald_press.f:413-419 */
        out->lj_pairs++;
    }
    if (el) {
        double rij = sqrt(r2), s = 1.0 / rij, erfcc, derfc;
        double q = in->ptchg[i - 1] * c->epstmp * in->ptchg[j - 1];
        erfc_pair(c, c->ewaldcof * rij, &erfcc, &derfc);
        e2 = q * s * erfcc;
        df2 = -q * s * (s2 * erfcc + s * c->ewaldcof * derfc);
        *eel += e2;
    }
    out->site_pairs++;
    df = df1 + df2;
    rx *= df; ry *= df; rz *= df;
    if (addi) { DP(0, i) += rx; DP(1, i) += ry; DP(2, i) += rz; }
    DP(0, j) -= rx; DP(1, j) -= ry; DP(2, j) -= rz;
}

/* One water-water molecule pair (watwat_ewald.f:131-612 list 1, :626-1089 list 2).
 * o_i is the i oxygen, sh the translation added to the i molecule. */
static void water_pair(const ctx *c, int list, int oi, int oj, const double sh[3],
                       double oosgm12, double oosgm6, const double qq[3][3],
                       double *dpot, double *evdw, double *eel, double *vir, ora_output *out)
{
    double xi[3][3], dfi[3][3] = {{0}};
    int a, b, k;
    double rx, ry, rz, r2;
    for (a = 0; a < 3; a++)
        for (k = 0; k < 3; k++) xi[a][k] = c->coor[3 * (oi + a - 1) + k] + sh[k];
    rx = xi[0][0] - X(oj); ry = xi[0][1] - Y(oj); rz = xi[0][2] - Z(oj);
    r2 = rx * rx + ry * ry + rz * rz;
    if (list == 2 && r2 > c->cutele2) return;
    out->site_pairs += 9;
    for (a = 0; a < 3; a++) {
        for (b = 0; b < 3; b++) {
            int j = oj + b;
            double dx = xi[a][0] - X(j), dy = xi[a][1] - Y(j), dz = xi[a][2] - Z(j);
            double rr2 = dx * dx + dy * dy + dz * dz, s2 = 1.0 / rr2;
            double rij = sqrt(rr2), s = 1.0 / rij, erfcc, derfc, df = 0, e2;
            if (list == 1 && a == 0 && b == 0 && rr2 <= c->cutvdw2) {
                double s6 = s2 * s2 * s2, aa = oosgm12 * s6 * s6, bb = oosgm6 * s6, e1 = aa - bb;
                df = -6.0 * s2 * (aa + e1);
                lj_switch(c, rr2, &e1, &df);
                *evdw += e1;
                *vir -= df * rr2;    /* watwat_ewald_press.f:146-152 (LJ part only) */
                out->lj_pairs++;
            }
            erfc_pair(c, c->ewaldcof * rij, &erfcc, &derfc);
            e2 = qq[a][b] * s * erfcc;
            df -= qq[a][b] * s * (s2 * erfcc + s * c->ewaldcof * derfc);
            *eel += e2;
            dx *= df; dy *= df; dz *= df;
            dfi[a][0] += dx; dfi[a][1] += dy; dfi[a][2] += dz;
            DP(0, j) -= dx; DP(1, j) -= dy; DP(2, j) -= dz;
        }
    }
    for (a = 0; a < 3; a++)
        for (k = 0; k < 3; k++) DP(k, oi + a) += dfi[a][k];
}

/* water constants from the last water (watwat_ewald.f:40-79) */
static void water_consts(const ctx *c, double *oosgm12, double *oosgm6, double qq[3][3])
{
    const ora_input *in = c->in;
    int m, io = 0, ih1;
    double qo, qh;
    for (m = in->totmon - 1; m >= 0; m--)
        if (c->iswat[m]) { io = in->poipt[m] - 2; break; }
    ih1 = io + 1;
    if (!in->arith) {
        *oosgm6 = in->epsgm6[io - 1] * in->epsgm6[io - 1];
        *oosgm12 = in->epsgm12[io - 1] * in->epsgm12[io - 1];
    } else {
        *oosgm6 = pow(in->epsgm12[io - 1], 2) * pow(in->epsgm6[io - 1], 6);
        *oosgm12 = pow(in->epsgm12[io - 1], 2) * pow(in->epsgm6[io - 1], 12);
    }
    qo = in->ptchg[io - 1]; qh = in->ptchg[ih1 - 1];
    qq[0][0] = c->epstmp * qo * qo;
    qq[0][1] = qq[0][2] = qq[1][0] = qq[2][0] = c->epstmp * qo * qh;
    qq[1][1] = qq[1][2] = qq[2][1] = qq[2][2] = c->epstmp * qh * qh;
}

/* cdie_ewald.f:117-199: erf corrections over the exclusion list (i < npt) */
static void excl_corr(const ctx *c, double *dpot, double *ecorr, ora_output *out)
{
    const ora_input *in = c->in;
    int i, k;
    for (i = 1; i <= in->npt - 1; i++) {
        double qi = in->ptchg[i - 1] * c->epstmp, dxi = 0, dyi = 0, dzi = 0;
        for (k = in->exc1[i - 1] + 1; k <= in->exc1[i]; k++) {
            int j = in->exc2[k - 1];
            double rx = X(i) - X(j), ry = Y(i) - Y(j), rz = Z(i) - Z(j);
            double r2 = rx * rx + ry * ry + rz * rz, s2 = 1.0 / r2, rij = sqrt(r2), s = 1.0 / rij;
            double q = qi * in->ptchg[j - 1], x = c->ewaldcof * rij, erfv, derfc, e2, df;
            if (in->erfc_mode == 0) {
                double erfcc = ora_erfc_table_eval(c->tab, c->erftbdns, x, &derfc);
                erfv = 1.0 - erfcc;
            } else {
                erfv = erf(x);
                derfc = 2.0 / sqrt(PI_D) * exp(-x * x);
            }
            e2 = -q * s * erfv;
            df = q * s * (s2 * erfv - s * c->ewaldcof * derfc);
            rx *= df; ry *= df; rz *= df;
            dxi += rx; dyi += ry; dzi += rz;
            DP(0, j) -= rx; DP(1, j) -= ry; DP(2, j) -= rz;
            *ecorr += e2;
            out->excl_pairs++;
        }
        DP(0, i) += dxi; DP(1, i) += dyi; DP(2, i) += dzi;
    }
}

/* ener14.f:38-95 */
static void ener14(const ctx *c, double *dpot, double *ev14, double *eel14, ora_output *out)
{
    const ora_input *in = c->in;
    int i;
    for (i = 0; i < in->totspe; i++) {
        int j = in->spec1[i], k = in->spec2[i];
        const double *p = in->p14 + 3 * i;
        double rx = X(j) - X(k), ry = Y(j) - Y(k), rz = Z(j) - Z(k);
        double r2 = rx * rx + ry * ry + rz * rz, s2 = 1.0 / r2, e1 = 0, df1 = 0, e2 = 0, df2 = 0, df;
        if (p[0] > 1e-12) {
            double s6 = s2 * s2 * s2, a = p[0] * s6 * s6, b = p[1] * s6;
            e1 = a - b;
            df1 = -6.0 * s2 * (a + e1);
            out->virvdw[4] -= df1 * r2;   /* ener14_press.f:51-59 */
        }
        if (fabs(p[2]) > 1e-12) {
            double s = sqrt(s2);
            e2 = p[2] * s;
            df2 = -e2 * s2;
        }
        df = df1 + df2;
        rx *= df; ry *= df; rz *= df;
        DP(0, j) += rx; DP(1, j) += ry; DP(2, j) += rz;
        DP(0, k) -= rx; DP(1, k) -= ry; DP(2, k) -= rz;
        *ev14 += e1; *eel14 += e2;
        out->n14++;
    }
}

static double self_energy(const ctx *c)
{
    /* ewald_init.f:131-150 */
    double s = 0;
    int i;
    for (i = 0; i < c->npt; i++) s += c->in->ptchg[i] * c->in->ptchg[i];
    return -c->ewaldcof * sqrt(1.0 / PI_D) * c->epstmp * s;
}

/* ------------------------------------------------------------------------ */
/* FFT (exact FP64 mixed radix; the MOIL FFTPACK result up to rounding)      */

/* Mixed-radix decimation-in-time DFT of length n (any n; small prime factors
 * first).  w holds exp(sign*2*pi*i*t/ntot) for t < ntot; a level of length n
 * uses every (ntot/n)-th entry. */
static void fft_rec(double *re, double *im, int n, const double *wr, const double *wi, int ntot,
                    double *tr, double *ti)
{
    int p, m, k, q, r;
    if (n == 1) return;
    for (p = 2; p * p <= n; p++) if (n % p == 0) break;
    if (n % p) p = n;
    m = n / p;
    for (r = 0; r < p; r++)
        for (k = 0; k < m; k++) {
            tr[r * m + k] = re[k * p + r];
            ti[r * m + k] = im[k * p + r];
        }
    for (r = 0; r < p; r++) fft_rec(tr + r * m, ti + r * m, m, wr, wi, ntot, re + r * m, im + r * m);
    {
        int step = ntot / n;
        for (k = 0; k < n; k++) {
            double sr = 0, si = 0;
            int kk = k % m;
            for (q = 0; q < p; q++) {
                int t = (int)(((long long)q * k) % n) * step;
                double cr = wr[t], ci = wi[t];
                double xr = tr[q * m + kk], xi = ti[q * m + kk];
                sr += xr * cr - xi * ci;
                si += xr * ci + xi * cr;
            }
            re[k] = sr;
            im[k] = si;
        }
    }
}

typedef struct fftplan { int n; double *wr, *wi, *tr, *ti, *lr, *li; } fftplan;

static void plan_init(fftplan *pl, int n, int sign)
{
    int t;
    pl->n = n;
    pl->wr = (double *)malloc(sizeof(double) * n); pl->wi = (double *)malloc(sizeof(double) * n);
    pl->tr = (double *)malloc(sizeof(double) * n); pl->ti = (double *)malloc(sizeof(double) * n);
    pl->lr = (double *)malloc(sizeof(double) * n); pl->li = (double *)malloc(sizeof(double) * n);
    for (t = 0; t < n; t++) {
        double ang = sign * 2.0 * PI_D * (double)t / n;
        pl->wr[t] = cos(ang);
        pl->wi[t] = sin(ang);
    }
}

static void plan_free(fftplan *pl)
{
    free(pl->wr); free(pl->wi); free(pl->tr); free(pl->ti); free(pl->lr); free(pl->li);
}

void ora_fft(double *re, double *im, int n, int sign)
{
    fftplan pl;
    plan_init(&pl, n, sign);
    fft_rec(re, im, n, pl.wr, pl.wi, n, pl.tr, pl.ti);
    plan_free(&pl);
}

static void fft3d(double *qr, double *qi, int n1, int n2, int n3, int sign)
{
    int i, j, k;
    fftplan p1, p2, p3;
    plan_init(&p1, n1, sign); plan_init(&p2, n2, sign); plan_init(&p3, n3, sign);
#define QI(i, j, k) ((size_t)(i) + (size_t)n1 * ((j) + (size_t)n2 * (k)))
    for (k = 0; k < n3; k++)
        for (j = 0; j < n2; j++) {
            double *lr = p1.lr, *li = p1.li;
            for (i = 0; i < n1; i++) { lr[i] = qr[QI(i, j, k)]; li[i] = qi[QI(i, j, k)]; }
            fft_rec(lr, li, n1, p1.wr, p1.wi, n1, p1.tr, p1.ti);
            for (i = 0; i < n1; i++) { qr[QI(i, j, k)] = lr[i]; qi[QI(i, j, k)] = li[i]; }
        }
    for (k = 0; k < n3; k++)
        for (i = 0; i < n1; i++) {
            double *lr = p2.lr, *li = p2.li;
            for (j = 0; j < n2; j++) { lr[j] = qr[QI(i, j, k)]; li[j] = qi[QI(i, j, k)]; }
            fft_rec(lr, li, n2, p2.wr, p2.wi, n2, p2.tr, p2.ti);
            for (j = 0; j < n2; j++) { qr[QI(i, j, k)] = lr[j]; qi[QI(i, j, k)] = li[j]; }
        }
    for (j = 0; j < n2; j++)
        for (i = 0; i < n1; i++) {
            double *lr = p3.lr, *li = p3.li;
            for (k = 0; k < n3; k++) { lr[k] = qr[QI(i, j, k)]; li[k] = qi[QI(i, j, k)]; }
            fft_rec(lr, li, n3, p3.wr, p3.wi, n3, p3.tr, p3.ti);
            for (k = 0; k < n3; k++) { qr[QI(i, j, k)] = lr[k]; qi[QI(i, j, k)] = li[k]; }
        }
#undef QI
    plan_free(&p1); plan_free(&p2); plan_free(&p3);
}

/* ------------------------------------------------------------------------ */
/* PME (pot/ewald_receip.f)                                                   */

/* fill_bspline / init / one_pass / diff (ewald_receip.f:1022-1080) */
static void fill_bspline(double w, int order, double *arr, double *darr)
{
    int k, j;
    arr[order - 1] = 0.0;
    arr[1] = w;
    arr[0] = 1.0 - w;
    for (k = 3; k <= order - 1; k++) {
        double div = 1.0 / (k - 1);
        arr[k - 1] = div * w * arr[k - 2];
        for (j = 1; j <= k - 2; j++)
            arr[k - j - 1] = div * ((w + j) * arr[k - j - 2] + (k - j - w) * arr[k - j - 1]);
        arr[0] = div * (1 - w) * arr[0];
    }
    darr[0] = -arr[0];
    for (j = 2; j <= order; j++) darr[j - 1] = arr[j - 2] - arr[j - 1];
    {
        double div = 1.0 / (order - 1);
        k = order;
        arr[k - 1] = div * w * arr[k - 2];
        for (j = 1; j <= k - 2; j++)
            arr[k - j - 1] = div * ((w + j) * arr[k - j - 2] + (k - j - w) * arr[k - j - 1]);
        arr[0] = div * (1 - w) * arr[0];
    }
}

/* load_bsp_moduli + DFTMOD (ewald_receip.f:413-481) */
int ora_bsp_moduli(int nfft, int order, double *mod)
{
    double arr[32], darr[32], *bsp;
    int j, k;
    if (order > 25) return -1;
    bsp = (double *)calloc(nfft + order + 2, sizeof(double));
    fill_bspline(0.0, order, arr, darr);
    for (j = 2; j <= order + 1 && j <= nfft; j++) bsp[j - 1] = arr[j - 2];
    for (k = 1; k <= nfft; k++) {
        double s1 = 0, s2 = 0;
        for (j = 1; j <= nfft; j++) {
            double arg = 2.0 * PI_D * (k - 1) * (j - 1) / nfft;
            s1 += bsp[j - 1] * cos(arg);
            s2 += bsp[j - 1] * sin(arg);
        }
        mod[k - 1] = s1 * s1 + s2 * s2;
    }
    for (k = 1; k <= nfft; k++)
        if (mod[k - 1] < 1e-7) {
            double lo = k > 1 ? mod[k - 2] : mod[nfft - 1];
            double hi = k < nfft ? mod[k] : mod[0];
            mod[k - 1] = 0.5 * (lo + hi);
        }
    free(bsp);
    return 0;
}

static int wrapidx(int k0, int n)
{
    /* k = k0 + 1 + (nfft - isign(nfft,k0))/2, as a 0-based index */
    int k = k0 >= 0 ? k0 : k0 + n;
    return k % n;   /* fr == nfft exactly lands on index 0 */
}

/* PME core; phi (nullable) receives dE_rec/dq per atom: fc * sum(theta * convolved grid).
 * press (nullable, with xrel): the pressure analysis terms, press[6..8] += the reciprocal
 * virial V_PIrec (ewald_receip.f:799-807) and press[9..11] += V_PIrel = sum of the PME force
 * times the atom's position relative to its molecule's centre of mass (:928-933). */
static int pme_core(const ora_input *in, double ewaldcof, double *dpot, double *eer, double *fpme_out, double *phi,
                    const double *xrel, double *press)
{
    int n1 = in->nfft1, n2 = in->nfft2, n3 = in->nfft3, order = in->order, N = in->npt;
    size_t ng = (size_t)n1 * n2 * n3;
    double *qr = (double *)calloc(ng, sizeof(double)), *qi = (double *)calloc(ng, sizeof(double));
    double *m1 = (double *)malloc(sizeof(double) * n1), *m2 = (double *)malloc(sizeof(double) * n2);
    double *m3 = (double *)malloc(sizeof(double) * n3);
    double *th = (double *)malloc(sizeof(double) * 6 * order * N);
    double *fr = (double *)malloc(sizeof(double) * 3 * N);
    double rc1 = 1.0 / in->a, rc2 = 1.0 / in->b, rc3 = 1.0 / in->c;
    double vol = in->a * in->b * in->c, epstmp = KOFDIE / in->eps, fc = sqrt(epstmp);
    double energy = 0, fpme = 0;
    int n, i1, i2, i3;
    ora_bsp_moduli(n1, order, m1);
    ora_bsp_moduli(n2, order, m2);
    ora_bsp_moduli(n3, order, m3);
#define Q(i, j, k) ((size_t)(i) + (size_t)n1 * ((j) + (size_t)n2 * (k)))
    /* get_scaled_fractionals (:250-260), get_bspline_coeffs (:973-1000) */
    for (n = 0; n < N; n++) {
        double w, *t = th + 6 * order * n;
        const double *x = in->coor + 3 * n;
        w = x[0] * rc1; fr[3 * n] = n1 * (w - round(w) + 0.5);
        w = x[1] * rc2; fr[3 * n + 1] = n2 * (w - round(w) + 0.5);
        w = x[2] * rc3; fr[3 * n + 2] = n3 * (w - round(w) + 0.5);
        fill_bspline(fr[3 * n] - (int)fr[3 * n], order, t, t + 3 * order);
        fill_bspline(fr[3 * n + 1] - (int)fr[3 * n + 1], order, t + order, t + 4 * order);
        fill_bspline(fr[3 * n + 2] - (int)fr[3 * n + 2], order, t + 2 * order, t + 5 * order);
    }
    /* fill_charge_grid (:600-711) */
    for (n = 0; n < N; n++) {
        const double *t = th + 6 * order * n;
        double fc1 = in->ptchg[n] * fc;
        int k0 = (int)fr[3 * n + 2] - order, j0b = (int)fr[3 * n + 1] - order, i0b = (int)fr[3 * n] - order;
        for (i3 = 0; i3 < order; i3++) {
            int k = wrapidx(++k0, n3), j0 = j0b;
            double prod = t[2 * order + i3] * fc1;
            for (i2 = 0; i2 < order; i2++) {
                int j = wrapidx(++j0, n2), i0 = i0b;
                double prod1 = t[order + i2] * prod;
                for (i1 = 0; i1 < order; i1++) {
                    int i = wrapidx(++i0, n1);
                    qr[Q(i, j, k)] += t[i1] * prod1;
                }
            }
        }
    }
    /* fft_back: isign = -1 */
    fft3d(qr, qi, n1, n2, n3, -1);
    /* scalar_sum (:723-812) */
    {
        double fac = PI_D * PI_D / (ewaldcof * ewaldcof), pivol = PI_D * vol;
        int nf1 = n1 / 2, nf2 = n2 / 2, nf3 = n3 / 2, k1, k2, k3;
        if (2 * nf1 < n1) nf1++;
        if (2 * nf2 < n2) nf2++;
        if (2 * nf3 < n3) nf3++;
        for (k3 = 1; k3 <= n3; k3++)
            for (k2 = 1; k2 <= n2; k2++)
                for (k1 = 1; k1 <= n1; k1++) {
                    int mm1 = k1 - 1, mm2 = k2 - 1, mm3 = k3 - 1;
                    double mh1, mh2, mh3, msq, denom, eterm, struc2;
                    size_t id = Q(k1 - 1, k2 - 1, k3 - 1);
                    if (k1 == 1 && k2 == 1 && k3 == 1) continue;
                    if (k1 > nf1) mm1 = k1 - 1 - n1;
                    if (k2 > nf2) mm2 = k2 - 1 - n2;
                    if (k3 > nf3) mm3 = k3 - 1 - n3;
                    mh1 = rc1 * mm1; mh2 = rc2 * mm2; mh3 = rc3 * mm3;
                    msq = mh1 * mh1 + mh2 * mh2 + mh3 * mh3;
                    denom = pivol * m1[k1 - 1] * m2[k2 - 1] * m3[k3 - 1] * msq;
                    eterm = exp(-fac * msq) / denom;
                    struc2 = qr[id] * qr[id] + qi[id] * qi[id];
                    energy += eterm * struc2;
                    if (press) {
                        double vp = 0.5 * eterm * struc2, b = 2.0 * (1.0 + fac * msq) / msq;
                        press[6] += vp * (1.0 - b * mh1 * mh1);
                        press[7] += vp * (1.0 - b * mh2 * mh2);
                        press[8] += vp * (1.0 - b * mh3 * mh3);
                    }
                    qr[id] *= eterm;
                    qi[id] *= eterm;
                }
        qr[0] = qi[0] = 0.0;   /* ind = 0 is skipped: m = 0 term left as is */
    }
    /* the m = 0 coefficient is untouched in MOIL; it multiplies no gradient
     * (sum of dtheta is zero), so zeroing it changes nothing below. */
    fft3d(qr, qi, n1, n2, n3, +1);
    /* grad_sum (:815-970) */
    for (n = 0; n < N; n++) {
        const double *t = th + 6 * order * n, *dt = t + 3 * order;
        double f1 = 0, f2 = 0, f3 = 0, term1 = fc * in->ptchg[n], fx, fy, fz;
        int k0 = (int)fr[3 * n + 2] - order, j0b = (int)fr[3 * n + 1] - order, i0b = (int)fr[3 * n] - order;
        for (i3 = 0; i3 < order; i3++) {
            int k = wrapidx(++k0, n3), j0 = j0b;
            double t3a = n3 * dt[2 * order + i3], t2a = n2 * t[2 * order + i3], t1a = n1 * t[2 * order + i3];
            for (i2 = 0; i2 < order; i2++) {
                int j = wrapidx(++j0, n2), i0 = i0b;
                double t3 = t3a * t[order + i2], t2 = t2a * dt[order + i2], t1 = t1a * t[order + i2];
                for (i1 = 0; i1 < order; i1++) {
                    int i = wrapidx(++i0, n1);
                    double term = term1 * qr[Q(i, j, k)];
                    f1 -= term * dt[i1] * t1;
                    f2 -= term * t[i1] * t2;
                    f3 -= term * t[i1] * t3;
                }
            }
        }
        fx = rc1 * f1; fy = rc2 * f2; fz = rc3 * f3;
        dpot[3 * n] -= fx; dpot[3 * n + 1] -= fy; dpot[3 * n + 2] -= fz;
        if (press) {
            press[9] += fx * xrel[3 * n];
            press[10] += fy * xrel[3 * n + 1];
            press[11] += fz * xrel[3 * n + 2];
        }
        if (phi) {
            double v = 0;
            k0 = (int)fr[3 * n + 2] - order;
            for (i3 = 0; i3 < order; i3++) {
                int k = wrapidx(++k0, n3), j0 = j0b;
                for (i2 = 0; i2 < order; i2++) {
                    int j = wrapidx(++j0, n2), i0 = i0b;
                    for (i1 = 0; i1 < order; i1++) {
                        int i = wrapidx(++i0, n1);
                        v += t[i1] * t[order + i2] * t[2 * order + i3] * qr[Q(i, j, k)];
                    }
                }
            }
            phi[n] += fc * v;
        }
        fpme += fx * fx + fy * fy + fz * fz;
    }
#undef Q
    *eer = 0.5 * energy;
    if (fpme_out) *fpme_out = sqrt(fpme / (3.0 * N));
    free(qr); free(qi); free(m1); free(m2); free(m3); free(th); free(fr);
    return 0;
}

int ora_pme(const ora_input *in, double ewaldcof, double *dpot, double *eer, double *fpme_out)
{
    return pme_core(in, ewaldcof, dpot, eer, fpme_out, 0, 0, 0);
}

/* ------------------------------------------------------------------------ */
/* eforce (pot/eforce.f:122-204) through MOIL's lists                         */

static void finish(ora_output *out)
{
    out->e_total = out->e_vdw + out->e_el + out->e_ew_receip + out->e_corr + out->e_self
                 + out->e_el14 + out->e_vdw14 + out->e_vsym + out->e_lsym;
    out->e_dir = out->e_el + out->e_lsym;
}

static void eforce_lists(ctx *c, lists *LL, double *dpot, ora_output *out);

int ora_eforce(const ora_input *in, double *dpot, ora_output *out)
{
    return ora_eforce_repeat(in, dpot, out, 1, 1);
}

/* nevals evaluations at the same coordinates with the lists rebuilt every
 * list_period evaluations: MOIL's dyna loop (dynamics/dyna.f:106-183) with '#lis'. */
int ora_eforce_repeat(const ora_input *in, double *dpot, ora_output *out, int nevals, int list_period)
{
    ctx cc, *c = &cc;
    lists L;
    int e;
    if (nevals < 1 || list_period < 1) return -2;
    if (ctx_init(c, in)) return -1;
    if (in->squeeze) squeeze(c);
    for (e = 0; e < nevals; e++) {
        if (e % list_period == 0) {
            if (e) free_lists(&L);
            build_lists(c, &L);
        }
        memset(out, 0, sizeof(*out));
        eforce_lists(c, &L, dpot, out);
    }
    free_lists(&L);
    ctx_free(c);
    return 0;
}

static void eforce_lists(ctx *c, lists *LL, double *dpot, ora_output *out)
{
    const ora_input *in = c->in;
    lists L = *LL;
    int i, k, isym;
    memset(dpot, 0, sizeof(double) * 3 * in->npt);
    out->ewaldcof = c->ewaldcof;
    out->e_self = self_energy(c);

    /* cdie_ewald: exclusion corrections, then list1/2/3 per atom i < npt */
    excl_corr(c, dpot, &out->e_corr, out);
    for (i = 1; i <= in->npt - 1; i++) {
        double xi = X(i), yi = Y(i), zi = Z(i);
        for (k = L.point1[i - 1] + 1; k <= L.point1[i]; k++)
            atom_pair(c, 1, i, xi, yi, zi, L.list1.v[k - 1], dpot, 1, &out->e_vdw, &out->e_el, &out->virvdw[2], out);
        for (k = L.point2[i - 1] + 1; k <= L.point2[i]; k++)
            atom_pair(c, 2, i, xi, yi, zi, L.list2.v[k - 1], dpot, 1, &out->e_vdw, &out->e_el, &out->virvdw[2], out);
        for (k = L.point3[i - 1] + 1; k <= L.point3[i]; k++)
            atom_pair(c, 3, i, xi, yi, zi, L.list3.v[k - 1], dpot, 1, &out->e_vdw, &out->e_el, &out->virvdw[2], out);
    }
    /* PME is periodic through anint (ewald_receip.f:250-260): squeezing does not change it */
    if (in->do_pme) ora_pme(in, c->ewaldcof, dpot, &out->e_ew_receip, &out->fpme);

    /* watwat_ewald (i = 1 .. nwaters-1) */
    if (L.nwaters > 1) {
        double o12, o6, qq[3][3], zero[3] = {0, 0, 0};
        int iw;
        water_consts(c, &o12, &o6, qq);
        for (iw = 1; iw <= L.nwaters - 1; iw++) {
            int oi = in->poipt[L.indxwat[iw]] - 2, kk;
            for (kk = L.poinwat1[iw] + 1; kk <= L.poinwat1[iw + 1]; kk++)
                water_pair(c, 1, oi, in->poipt[L.listwt1.v[kk - 1]] - 2, zero, o12, o6, qq, dpot,
                           &out->e_vdw, &out->e_el, &out->virvdw[0], out);
            for (kk = L.poinwat2[iw] + 1; kk <= L.poinwat2[iw + 1]; kk++)
                water_pair(c, 2, oi, in->poipt[L.listwt2.v[kk - 1]] - 2, zero, o12, o6, qq, dpot,
                           &out->e_vdw, &out->e_el, &out->virvdw[0], out);
        }
    }
    /* ener14 */
    ener14(c, dpot, &out->e_vdw14, &out->e_el14, out);

    /* symcdie_ewald: list1/2/3 image blocks */
    {
        long long jb1 = L.nprim1 + 1, jb2 = L.nprim2 + 1, jb3 = L.nprim3 + 1;
        int is1 = 1, is2 = 1, is3 = 1;
        for (isym = 1; isym <= 13; isym++) {
            double sh[3];
            int ii;
            for (k = 0; k < 3; k++) sh[k] = L.symop[isym - 1][k] * (k == 0 ? in->a : k == 1 ? in->b : in->c);
            for (ii = is1; ii <= L.iblock1[isym]; ii++) {
                int ir = L.symreal1.v[ii - 1], je = L.psym1.v[ii - 1];
                for (k = (int)jb1; k <= je; k++)
                    atom_pair(c, 1, ir, X(ir) + sh[0], Y(ir) + sh[1], Z(ir) + sh[2], L.list1.v[k - 1], dpot, 1,
                              &out->e_vsym, &out->e_lsym, &out->virvdw[3], out);
                jb1 = je + 1;
            }
            is1 = L.iblock1[isym] + 1;
            for (ii = is2; ii <= L.iblock2[isym]; ii++) {
                int ir = L.symreal2.v[ii - 1], je = L.psym2.v[ii - 1];
                for (k = (int)jb2; k <= je; k++)
                    atom_pair(c, 2, ir, X(ir) + sh[0], Y(ir) + sh[1], Z(ir) + sh[2], L.list2.v[k - 1], dpot, 1,
                              &out->e_vsym, &out->e_lsym, &out->virvdw[3], out);
                jb2 = je + 1;
            }
            is2 = L.iblock2[isym] + 1;
            for (ii = is3; ii <= L.iblock3[isym]; ii++) {
                int ir = L.symreal3.v[ii - 1], je = L.psym3.v[ii - 1];
                for (k = (int)jb3; k <= je; k++)
                    atom_pair(c, 3, ir, X(ir) + sh[0], Y(ir) + sh[1], Z(ir) + sh[2], L.list3.v[k - 1], dpot, 1,
                              &out->e_vsym, &out->e_lsym, &out->virvdw[3], out);
                jb3 = je + 1;
            }
            is3 = L.iblock3[isym] + 1;
        }
    }
    /* symwat_ewald: water image blocks */
    if (L.nwaters > 0) {
        double o12, o6, qq[3][3];
        long long jb1 = L.nprimw1 + 1, jb2 = L.nprimw2 + 1;
        int is1 = 1, is2 = 1;
        water_consts(c, &o12, &o6, qq);
        for (isym = 1; isym <= 13; isym++) {
            double sh[3];
            int ii;
            for (k = 0; k < 3; k++) sh[k] = L.symop[isym - 1][k] * (k == 0 ? in->a : k == 1 ? in->b : in->c);
            for (ii = is1; ii <= L.iblckwt1[isym]; ii++) {
                int oi = in->poipt[L.symmwat1.v[ii - 1]] - 2, je = L.psymwt1.v[ii - 1];
                for (k = (int)jb1; k <= je; k++)
                    water_pair(c, 1, oi, in->poipt[L.listwt1.v[k - 1]] - 2, sh, o12, o6, qq, dpot,
                               &out->e_vsym, &out->e_lsym, &out->virvdw[1], out);
                jb1 = je + 1;
            }
            is1 = L.iblckwt1[isym] + 1;
            for (ii = is2; ii <= L.iblckwt2[isym]; ii++) {
                int oi = in->poipt[L.symmwat2.v[ii - 1]] - 2, je = L.psymwt2.v[ii - 1];
                for (k = (int)jb2; k <= je; k++)
                    water_pair(c, 2, oi, in->poipt[L.listwt2.v[k - 1]] - 2, sh, o12, o6, qq, dpot,
                               &out->e_vsym, &out->e_lsym, &out->virvdw[1], out);
                jb2 = je + 1;
            }
            is2 = L.iblckwt2[isym] + 1;
        }
    }
    out->list_sizes[0] = L.list1.n; out->list_sizes[1] = L.list2.n; out->list_sizes[2] = L.list3.n;
    out->list_sizes[3] = L.listwt1.n; out->list_sizes[4] = L.listwt2.n;
    out->list_sizes[5] = L.nprim1; out->list_sizes[6] = L.nprimw1; out->list_sizes[7] = L.nprimw2;
    finish(out);
}

/* ------------------------------------------------------------------------ */
/* independent minimum-image evaluator (exact predicate at the coordinates)  */

typedef struct cellgrid {
    int nc[3];
    double inv[3];
    int *head, *next;
} cellgrid;

/* Minimum-image evaluation; with xrel (positions relative to the molecules' centres of
 * mass) it also accumulates the pressure analysis terms into press[12] (see ora_pressure_mi). */
static int eforce_mi_core(const ora_input *in, double *dpot, ora_output *out, const double *xrel, double *press)
{
    ctx cc, *c = &cc;
    int npt = in->npt, i, m;
    int *mol, *oxy;            /* per atom: monomer, water oxygen (1-based) or 0 */
    char **exset = 0;
    double box[3] = {in->a, in->b, in->c};
    double rmax2, rcut_el2, o12 = 0, o6 = 0, qq[3][3];
    int has_water = 0;
    memset(out, 0, sizeof(*out));
    if (ctx_init(c, in)) return -1;
    memset(dpot, 0, sizeof(double) * 3 * npt);
    out->ewaldcof = c->ewaldcof;
    out->e_self = self_energy(c);
    mol = (int *)malloc(sizeof(int) * (npt + 1));
    oxy = (int *)calloc(npt + 1, sizeof(int));
    for (m = 0; m < in->totmon; m++)
        for (i = c->first[m]; i <= in->poipt[m]; i++) {
            mol[i] = m;
            if (c->iswat[m]) { oxy[i] = in->poipt[m] - 2; has_water = 1; }
        }
    if (has_water) water_consts(c, &o12, &o6, qq);
    (void)exset;
    rcut_el2 = c->cutele2 > c->cutvdw2 ? c->cutele2 : c->cutvdw2;
    rmax2 = rcut_el2;
    excl_corr(c, dpot, &out->e_corr, out);
    ener14(c, dpot, &out->e_vdw14, &out->e_el14, out);
    if (in->do_pme) pme_core(in, c->ewaldcof, dpot, &out->e_ew_receip, &out->fpme, 0, xrel, press);
    {
        /* cell list over atoms; cell edge >= cutoff + 2 Å (water site offsets) */
        double reach = sqrt(rmax2) + 2.2;
        int d, nc[3], ncell;
        int *head, *next;
        for (d = 0; d < 3; d++) { nc[d] = (int)floor(box[d] / reach); if (nc[d] < 1) nc[d] = 1; }
        ncell = nc[0] * nc[1] * nc[2];
        head = (int *)malloc(sizeof(int) * ncell);
        next = (int *)malloc(sizeof(int) * (npt + 1));
        for (i = 0; i < ncell; i++) head[i] = 0;
        for (i = npt; i >= 1; i--) {
            int cidx[3], q;
            for (d = 0; d < 3; d++) {
                double x = c->coor[3 * (i - 1) + d];
                double f = x / box[d] + 0.5;
                f -= floor(f);
                q = (int)(f * nc[d]);
                if (q >= nc[d]) q = nc[d] - 1;
                cidx[d] = q;
            }
            q = cidx[0] + nc[0] * (cidx[1] + nc[1] * cidx[2]);
            next[i] = head[q];
            head[q] = i;
        }
        for (i = 1; i <= npt; i++) {
            int ci[3], dx, dy, dz, q;
            int offs[3][3], no[3];
            for (d = 0; d < 3; d++) {
                double f = c->coor[3 * (i - 1) + d] / box[d] + 0.5;
                f -= floor(f);
                q = (int)(f * nc[d]);
                if (q >= nc[d]) q = nc[d] - 1;
                ci[d] = q;
                /* unique neighbour cells along d */
                no[d] = 0;
                {
                    int t, u, dup;
                    for (t = -1; t <= 1; t++) {
                        int v = ((ci[d] + t) % nc[d] + nc[d]) % nc[d];
                        dup = 0;
                        for (u = 0; u < no[d]; u++) if (offs[d][u] == v) dup = 1;
                        if (!dup) offs[d][no[d]++] = v;
                    }
                }
            }
            for (dz = 0; dz < no[2]; dz++)
                for (dy = 0; dy < no[1]; dy++)
                    for (dx = 0; dx < no[0]; dx++) {
                        int j = head[offs[0][dx] + nc[0] * (offs[1][dy] + nc[1] * offs[2][dz])];
                        for (; j; j = next[j]) {
                            double rv[3], sh[3], r2 = 0, img = 0;
                            int ww = 0, k;
                            if (j <= i) continue;
                            if (oxy[i] && oxy[j] && mol[i] != mol[j]) {
                                ww = 1;
                                for (k = 0; k < 3; k++) {
                                    double a = c->coor[3 * (oxy[i] - 1) + k] - c->coor[3 * (oxy[j] - 1) + k];
                                    sh[k] = box[k] * round(a / box[k]);
                                    r2 += (a - sh[k]) * (a - sh[k]);
                                    img += fabs(sh[k]);
                                }
                                if (r2 > rcut_el2) continue;
                            } else {
                                if (excluded(in, i, j)) continue;
                                if (oxy[i] && oxy[j]) continue;   /* same water */
                                for (k = 0; k < 3; k++) {
                                    double a = c->coor[3 * (i - 1) + k] - c->coor[3 * (j - 1) + k];
                                    sh[k] = box[k] * round(a / box[k]);
                                    r2 += (a - sh[k]) * (a - sh[k]);
                                    img += fabs(sh[k]);
                                }
                                if (r2 >= rmax2 && !(r2 < c->cutvdw2)) continue;
                            }
                            for (k = 0; k < 3; k++) rv[k] = c->coor[3 * (i - 1) + k] - c->coor[3 * (j - 1) + k] - sh[k];
                            {
                                double rr2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
                                double s2 = 1.0 / rr2, e1 = 0, df1 = 0, e2 = 0, df2 = 0, df;
                                int lj, el;
                                double *ev = img > 0 ? &out->e_vsym : &out->e_vdw;
                                double *ee = img > 0 ? &out->e_lsym : &out->e_el;
                                double *vv = &out->virvdw[(ww ? 0 : 2) + (img > 0)];
                                if (ww) {
                                    int a = i - oxy[i], b = j - oxy[j];
                                    lj = (a == 0 && b == 0) && rr2 <= c->cutvdw2;
                                    el = 1;
                                    if (lj) {
                                        double s6 = s2 * s2 * s2, aa = o12 * s6 * s6, bb = o6 * s6;
                                        e1 = aa - bb;
                                        df1 = -6.0 * s2 * (aa + e1);
                                    }
                                    if (el) {
                                        double rij = sqrt(rr2), s = 1.0 / rij, erfcc, derfc;
                                        erfc_pair(c, c->ewaldcof * rij, &erfcc, &derfc);
                                        e2 = qq[a][b] * s * erfcc;
                                        df2 = -qq[a][b] * s * (s2 * erfcc + s * c->ewaldcof * derfc);
                                    }
                                } else {
                                    int hr = (!in->arith) && in->hvdw0 && rr2 < c->cutele2 &&
                                             (in->epsgm12[i - 1] < 1e-3 || in->epsgm12[j - 1] < 1e-3);
                                    int both = c->flagchr[i - 1] && c->flagchr[j - 1];
                                    lj = rr2 < c->cutvdw2 && !hr;
                                    el = both && (rr2 < rcut_el2);
                                    if (!lj && !el) continue;
                                    if (lj) {
                                        double a, b;
                                        lj_ab(c, i, j, s2, &a, &b);
                                        e1 = a - b;
                                        df1 = -6.0 * s2 * (a + e1);
                                    }
                                    if (el) {
                                        double rij = sqrt(rr2), s = 1.0 / rij, erfcc, derfc;
                                        double q = in->ptchg[i - 1] * c->epstmp * in->ptchg[j - 1];
                                        erfc_pair(c, c->ewaldcof * rij, &erfcc, &derfc);
                                        e2 = q * s * erfcc;
                                        df2 = -q * s * (s2 * erfcc + s * c->ewaldcof * derfc);
                                    }
                                }
                                if (lj) { lj_switch(c, rr2, &e1, &df1); out->lj_pairs++; *vv -= df1 * rr2; }
                                out->site_pairs++;
                                *ev += e1;
                                *ee += e2;
                                df = df1 + df2;
                                for (k = 0; k < 3; k++) {
                                    dpot[3 * (i - 1) + k] += df * rv[k];
                                    dpot[3 * (j - 1) + k] -= df * rv[k];
                                }
                                if (press)
                                    for (k = 0; k < 3; k++) {
                                        /* centre-of-mass separation of the two molecules, in
                                         * the image this pair is taken in */
                                        double rm = rv[k] - xrel[3 * (i - 1) + k] + xrel[3 * (j - 1) + k];
                                        press[k] -= df1 * rv[k] * rm;       /* virXX..ZZ */
                                        press[3 + k] -= df2 * rv[k] * rm;   /* V_PIdirXX..ZZ */
                                    }
                            }
                        }
                    }
        }
        free(head); free(next);
    }
    finish(out);
    free(mol); free(oxy);
    ctx_free(c);
    return 0;
}

int ora_eforce_mi(const ora_input *in, double *dpot, ora_output *out)
{
    return eforce_mi_core(in, dpot, out, 0, 0);
}

/* Positions relative to the molecules' centres of mass (analysis/pressure.f: checkANDmove
 * :985-1010 makes each molecule whole along its bonds, atom2molecule :419-520 forms the
 * centres of mass).  Here each atom is placed at the minimum image of its displacement
 * from the previous atom of its molecule in atom order, which makes the molecule whole
 * whenever consecutive atoms of a molecule are closer than half the box. */
static int mol_xrel(const ora_input *in, const int *mol, const double *mass, double *xrel)
{
    int n, k, m, nm = 0, npt = in->npt;
    double box[3] = {in->a, in->b, in->c};
    int *last;
    double *msum, *mds;
    for (n = 0; n < npt; n++) {
        if (mol[n] < 0) return -1;
        if (mol[n] + 1 > nm) nm = mol[n] + 1;
    }
    last = (int *)malloc(sizeof(int) * (nm + 1));
    msum = (double *)calloc(nm + 1, sizeof(double));
    mds = (double *)calloc(3 * (size_t)(nm + 1), sizeof(double));
    for (m = 0; m < nm; m++) last[m] = -1;
    for (n = 0; n < npt; n++) {
        m = mol[n];
        for (k = 0; k < 3; k++) {
            double d = 0.0;
            if (last[m] >= 0) {
                double t = in->coor[3 * n + k] - in->coor[3 * last[m] + k];
                d = xrel[3 * last[m] + k] + t - box[k] * round(t / box[k]);
            }
            xrel[3 * n + k] = d;
            mds[3 * m + k] += mass[n] * d;
        }
        msum[m] += mass[n];
        last[m] = n;
    }
    for (n = 0; n < npt; n++) {
        m = mol[n];
        for (k = 0; k < 3; k++) xrel[3 * n + k] -= msum[m] > 0.0 ? mds[3 * m + k] / msum[m] : 0.0;
    }
    free(last); free(msum); free(mds);
    return 0;
}

int ora_pressure_mi(const ora_input *in, const int *mol, const double *mass, double *dpot, ora_output *out,
                    double *press)
{
    double *xrel = (double *)malloc(sizeof(double) * 3 * (size_t)(in->npt > 0 ? in->npt : 1));
    int k, rc;
    for (k = 0; k < 12; k++) press[k] = 0.0;
    rc = mol_xrel(in, mol, mass, xrel);
    if (rc == 0) rc = eforce_mi_core(in, dpot, out, xrel, press);
    free(xrel);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Parameter derivatives (no MOIL counterpart; pinned by finite differences of the energy):
 * dE/dq_i (the electrostatic potential at i), dE/deps_i and dE/dsigma_i of atom i's LJ
 * parameters, decoded from the epsgm encoding (connect/fillpt.f:136-184).  Same pair
 * predicate as ora_eforce_mi; the LJ switch is not applied.  Water-water charge products
 * use each site's own charge (MOIL uses the last water's, equal for identical waters). */
static void lj_decode(const ora_input *in, int i, double *eps, double *sig)
{
    double e12 = in->epsgm12[i], e6 = in->epsgm6[i];
    if (!in->arith) {
        if (e12 > 0 && e6 > 0) {
            double se = e6 * e6 / (2.0 * e12);   /* sqrt(eps): epsgm6 = 2 sqrt(eps) sigma^3 */
            *sig = cbrt(e12 / e6);                /* epsgm12 / epsgm6 = sigma^3 */
            *eps = se * se;
        } else {
            *eps = 0; *sig = 0;
        }
    } else {
        *eps = 0.25 * e12 * e12;                  /* epsgm12 = 2 sqrt(eps) */
        *sig = e6;                                /* epsgm6 = sigma */
    }
}

/* pair LJ energy e = a - b (a ~ r^-12, b ~ r^-6 parts) into atoms i, j (0-based) */
static void lj_adjoint(const ora_input *in, int i, int j, double a, double b, const double *eps,
                       const double *sig, double *de, double *ds)
{
    double e = a - b, g = 6.0 * a - 3.0 * b;
    if (de) {
        if (eps[i] > 0) de[i] += e / (2.0 * eps[i]);
        if (eps[j] > 0) de[j] += e / (2.0 * eps[j]);
    }
    if (ds) {
        if (!in->arith) {
            if (sig[i] > 0) ds[i] += g / sig[i];
            if (sig[j] > 0) ds[j] += g / sig[j];
        } else {
            double sij = 0.5 * (sig[i] + sig[j]);
            if (sij > 0) { ds[i] += g / sij; ds[j] += g / sij; }
        }
    }
}

int ora_adjoint_mi(const ora_input *in, double *dq, double *de, double *ds)
{
    ctx cc, *c = &cc;
    int npt = in->npt, i, m, k;
    int *mol, *oxy;
    double box[3] = {in->a, in->b, in->c};
    double rcut_el2, o12 = 0, o6 = 0, qq[3][3];
    double *eps, *sig, *dpot;
    int has_water = 0;
    if (ctx_init(c, in)) return -1;
    if (dq) memset(dq, 0, sizeof(double) * npt);
    if (de) memset(de, 0, sizeof(double) * npt);
    if (ds) memset(ds, 0, sizeof(double) * npt);
    eps = (double *)malloc(sizeof(double) * npt);
    sig = (double *)malloc(sizeof(double) * npt);
    for (i = 0; i < npt; i++) lj_decode(in, i, eps + i, sig + i);
    mol = (int *)malloc(sizeof(int) * (npt + 1));
    oxy = (int *)calloc(npt + 1, sizeof(int));
    for (m = 0; m < in->totmon; m++)
        for (i = c->first[m]; i <= in->poipt[m]; i++) {
            mol[i] = m;
            if (c->iswat[m]) { oxy[i] = in->poipt[m] - 2; has_water = 1; }
        }
    if (has_water) water_consts(c, &o12, &o6, qq);
    rcut_el2 = c->cutele2 > c->cutvdw2 ? c->cutele2 : c->cutvdw2;
    /* self energy (ewald_init.f:131-150) and PME potential */
    if (dq) {
        for (i = 0; i < npt; i++) dq[i] += -2.0 * c->ewaldcof * sqrt(1.0 / PI_D) * c->epstmp * in->ptchg[i];
        if (in->do_pme) {
            double eer;
            dpot = (double *)calloc(3 * (size_t)npt, sizeof(double));
            pme_core(in, c->ewaldcof, dpot, &eer, 0, dq, 0, 0);
            free(dpot);
        }
    }
    /* exclusion corrections (cdie_ewald.f:117-199) */
    for (i = 1; i <= npt - 1; i++)
        for (k = in->exc1[i - 1] + 1; k <= in->exc1[i]; k++) {
            int j = in->exc2[k - 1];
            double rx = X(i) - X(j), ry = Y(i) - Y(j), rz = Z(i) - Z(j);
            double rij = sqrt(rx * rx + ry * ry + rz * rz), f;
            if (!dq) continue;
            f = -c->epstmp * erf(c->ewaldcof * rij) / rij;
            dq[i - 1] += f * in->ptchg[j - 1];
            dq[j - 1] += f * in->ptchg[i - 1];
        }
    /* 1-4 (ener14.f:38-95): p14(3) = q_j q_k kofdie el14 / eps */
    for (k = 0; k < in->totspe; k++) {
        int j = in->spec1[k], l = in->spec2[k];
        const double *p = in->p14 + 3 * k;
        double rx = X(j) - X(l), ry = Y(j) - Y(l), rz = Z(j) - Z(l);
        double r2 = rx * rx + ry * ry + rz * rz, s2 = 1.0 / r2, s6 = s2 * s2 * s2, s = sqrt(s2);
        if (p[0] > 1e-12) lj_adjoint(in, j - 1, l - 1, p[0] * s6 * s6, p[1] * s6, eps, sig, de, ds);
        if (dq && fabs(p[2]) > 1e-12) {
            if (fabs(in->ptchg[j - 1]) > 1e-12) dq[j - 1] += p[2] / in->ptchg[j - 1] * s;
            if (fabs(in->ptchg[l - 1]) > 1e-12) dq[l - 1] += p[2] / in->ptchg[l - 1] * s;
        }
    }
    /* real space: all pairs, minimum image */
    for (i = 1; i <= npt; i++) {
        int j;
        for (j = i + 1; j <= npt; j++) {
            double rv[3], sh[3], r2 = 0, rr2, s2, s6;
            int ww = 0;
            if (oxy[i] && oxy[j] && mol[i] != mol[j]) {
                ww = 1;
                for (k = 0; k < 3; k++) {
                    double a = c->coor[3 * (oxy[i] - 1) + k] - c->coor[3 * (oxy[j] - 1) + k];
                    sh[k] = box[k] * round(a / box[k]);
                    r2 += (a - sh[k]) * (a - sh[k]);
                }
                if (r2 > rcut_el2) continue;
            } else {
                if (excluded(in, i, j)) continue;
                if (oxy[i] && oxy[j]) continue;   /* same water */
                for (k = 0; k < 3; k++) {
                    double a = c->coor[3 * (i - 1) + k] - c->coor[3 * (j - 1) + k];
                    sh[k] = box[k] * round(a / box[k]);
                    r2 += (a - sh[k]) * (a - sh[k]);
                }
                if (r2 >= rcut_el2 && !(r2 < c->cutvdw2)) continue;
            }
            for (k = 0; k < 3; k++) rv[k] = c->coor[3 * (i - 1) + k] - c->coor[3 * (j - 1) + k] - sh[k];
            rr2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
            s2 = 1.0 / rr2;
            s6 = s2 * s2 * s2;
            if (ww) {
                int a = i - oxy[i], b = j - oxy[j];
                double rij = sqrt(rr2), f = c->epstmp * erfc(c->ewaldcof * rij) / rij;
                if (a == 0 && b == 0 && rr2 <= c->cutvdw2) lj_adjoint(in, i - 1, j - 1, o12 * s6 * s6, o6 * s6, eps, sig, de, ds);
                if (dq) { dq[i - 1] += f * in->ptchg[j - 1]; dq[j - 1] += f * in->ptchg[i - 1]; }
            } else {
                int hr = (!in->arith) && in->hvdw0 && rr2 < c->cutele2 &&
                         (in->epsgm12[i - 1] < 1e-3 || in->epsgm12[j - 1] < 1e-3);
                int both = c->flagchr[i - 1] && c->flagchr[j - 1];
                if (rr2 < c->cutvdw2 && !hr) {
                    double a, b;
                    lj_ab(c, i, j, s2, &a, &b);
                    lj_adjoint(in, i - 1, j - 1, a, b, eps, sig, de, ds);
                }
                if (both && rr2 < rcut_el2 && dq) {
                    double rij = sqrt(rr2), f = c->epstmp * erfc(c->ewaldcof * rij) / rij;
                    dq[i - 1] += f * in->ptchg[j - 1];
                    dq[j - 1] += f * in->ptchg[i - 1];
                }
            }
        }
    }
    free(eps); free(sig); free(mol); free(oxy);
    ctx_free(c);
    return 0;
}

int ora_eforce_batch(int nsys, const ora_input *in, double **dpot, ora_output *out, int mi, int nthreads,
                     int nevals, int list_period)
{
    int s, bad = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : bad)
#endif
    for (s = 0; s < nsys; s++) {
        int r = mi ? ora_eforce_mi(&in[s], dpot[s], &out[s])
                   : ora_eforce_repeat(&in[s], dpot[s], &out[s], nevals, list_period);
        if (r) bad++;
    }
    (void)nthreads;
    return bad ? -1 : 0;
}

/*
 * moil_oracle.h -- CPU FP64 restatement of MOIL's nonbonded Ewald path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against; nothing in the product links, loads or calls it.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark use it.
 *
 * Every routine follows a MOIL source file (paths relative to the MOIL tree):
 *   ora_find_ewaldcof      symm/ewald_init.f:298-335
 *   erfc spline table      symm/ewald_init.f:101-126, 418-574 (de Boor cubspl)
 *   self energy            symm/ewald_init.f:131-150
 *   B-spline moduli        pot/ewald_receip.f:413-481
 *   squeeze                symm/squeeze.f:66-145
 *   monomer lists          pot/nbondm.f:79-241
 *   atom lists             pot/nbond.f:54-157
 *   image lists            symm/syminit.f:80-164, symm/nbmsym.f, symm/nbsym.f
 *   exclusion corrections  pot/cdie_ewald.f:117-199
 *   list1/list2/list3      pot/cdie_ewald.f:313-671
 *   water-water            pot/watwat_ewald.f:40-1104
 *   1-4                    pot/ener14.f:38-95
 *   image kernels          symm/symcdie_ewald.f:63-467, symm/symwat_ewald.f:88-1133
 *   PME                    pot/ewald_receip.f:101-1080
 *   composition            pot/eforce.f:122-204
 */
#ifndef MOIL_ORACLE_H
#define MOIL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_input {
    int npt;
    const double *coor;      /* npt*3, coor(3,npt) */
    const double *ptchg;     /* npt */
    const double *epsgm6;    /* npt */
    const double *epsgm12;   /* npt */
    const int *exc1;         /* npt+1, exc1(0:npt) */
    const int *exc2;         /* exc1[npt], 1-based */
    int totspe;
    const int *spec1, *spec2;/* 1-based */
    const double *p14;       /* totspe*3, p14(3,totspe) */
    int totmon;
    const int *poipt;        /* 1-based last atom of each monomer */
    const int *montype;      /* 0 other, 1 water, 2 squeezed ion */
    int arith, hvdw0;
    double a, b, c;          /* box */
    double rvmx, rvbg, relx, rebg, cutm;  /* Å; rvbg/rebg < 0 -> +2 Å, cutm < 0 -> 1.2*rebg */
    double eps;              /* dielectric */
    double ewaldcof;         /* > 0: use as is; otherwise from dtol */
    double dtol;
    int nfft1, nfft2, nfft3, order;
    int erfc_mode;           /* 0: MOIL cubic-spline table, 1: exact erfc */
    int lj_switch;           /* extension (not in MOIL): CHARMM LJ switch on [r_on, rvmx] */
    double r_on;
    int squeeze;             /* 1: wrap water/ion monomers as symm/squeeze.f does */
    int do_pme;              /* 1: include ewald_receip */
} ora_input;

typedef struct ora_output {
    double e_vdw, e_el, e_vsym, e_lsym, e_el14, e_vdw14;
    double e_corr, e_self, e_ew_receip, e_total, e_dir;
    double ewaldcof;
    double fpme;
    long long site_pairs;    /* site pairs evaluated inside the cutoff predicate */
    long long lj_pairs;      /* of those, pairs with an LJ term */
    long long excl_pairs;    /* exclusion-correction pairs */
    long long n14;           /* 1-4 pairs */
    long long list_sizes[8]; /* list1,list2,list3,listwt1,listwt2 (primary + images) */
    /* LJ virial terms of MOIL's PRESS build (pot/watwat_ewald_press.f:146-152,
     * symm/symwat_ewald_press.f:161-168, pot/cdie_ewald_press.f:413-419,
     * symm/symcdie_ewald_press.f:164-167, pot/ener14_press.f:51-59): virvdw = -sum df1 r^2
     * over the LJ pairs (df1 = (dE/dr)/r of the LJ part) of water-water primary, water-water
     * images, other primary, other images, and 1-4 pairs */
    double virvdw[5];
} ora_output;

/* MOIL path: squeeze (optional) -> nbondm/nbond -> syminit -> eforce nonbonded block. */
int ora_eforce(const ora_input *in, double *dpot, ora_output *out);

/* Independent minimum-image evaluation with MOIL's pair predicate applied exactly
 * at the given coordinates (the parity reference for the GPU path). */
int ora_eforce_mi(const ora_input *in, double *dpot, ora_output *out);

/* MOIL's pressure analysis terms (analysis/pressure.f with pressON) at the given coordinates,
 * beside the ora_eforce_mi evaluation.  mol[n]: molecule of atom n (0-based ids), mass[n]:
 * its mass.  press[12] = virXX, virYY, virZZ (LJ, watwat_ewald.f:163-175, cdie_ewald.f:
 * 441-453, 555-566), V_PIdirXX..ZZ (real-space Ewald Coulomb, watwat_ewald.f:196-204,
 * cdie_ewald.f:412-429), V_PIrecXX..ZZ (reciprocal, ewald_receip.f:799-807), V_PIrelXX..ZZ
 * (PME force times the position relative to the centre of mass, ewald_receip.f:928-933):
 * every pair term is F_ij,a (R_I - R_J)_a with R the molecules' centres of mass in the image
 * the pair is taken in; pressure.f:235-238 sums vir + dir + rec - rel (V_PIcor is zero:
 * its accumulation is commented out in cdie_ewald.f:165-170). */
int ora_pressure_mi(const ora_input *in, const int *mol, const double *mass, double *dpot, ora_output *out,
                    double *press);

/* nevals evaluations with lists rebuilt every list_period (MOIL's '#lis'). */
int ora_eforce_repeat(const ora_input *in, double *dpot, ora_output *out, int nevals, int list_period);

/* Parameter derivatives at the given coordinates (arrays of npt, any may be NULL): dE/dq,
 * dE/deps and dE/dsigma per atom, LJ parameters decoded from the epsgm encoding. */
int ora_adjoint_mi(const ora_input *in, double *dEdq, double *dEdeps, double *dEdsig);

/* Batch of independent systems, OpenMP over systems (CPU baseline); mi selects the
 * minimum-image evaluator, otherwise nevals/list_period as ora_eforce_repeat. */
int ora_eforce_batch(int nsys, const ora_input *in, double **dpot, ora_output *out, int mi, int nthreads,
                     int nevals, int list_period);

double ora_find_ewaldcof(double cutoff, double dtol);
/* erfc table: returns number of points (4 coefficients each) written to tab (capacity cap). */
int ora_erfc_table(double ewaldcof, double cutoff, double *tab, int cap);
double ora_erfc_table_eval(const double *tab, double erftbdns, double x, double *derfc);
int ora_bsp_moduli(int nfft, int order, double *mod);
/* PME reciprocal energy/forces alone (adds to dpot). */
int ora_pme(const ora_input *in, double ewaldcof, double *dpot, double *eer, double *fpme);
/* In-place complex FFT of length n (sign -1 or +1), unnormalised, stride 1. */
void ora_fft(double *re, double *im, int n, int sign);

#ifdef __cplusplus
}
#endif
#endif

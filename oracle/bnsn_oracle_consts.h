/* Test infrastructure only: physical constants of the bns_nurates opacity path,
 * restated for the CPU oracle.  Every derived value is written as the same
 * double-precision expression the reference evaluates
 * (include/constants.hpp:30-244), so the folded values are identical.
 */
#ifndef BNSN_ORACLE_CONSTS_H_
#define BNSN_ORACLE_CONSTS_H_

#define SQ(X) ((X) * (X))
#define CUBE(X) ((X) * (X) * (X))

/* constants.hpp:30-90 */
#define C_MEV 1.6021766341182763e+8
#define C_ME 0.51099895069
#define C_MN 939.56542194
#define C_MP 938.27208943
#define C_Q 1.29333251
#define C_MU 1.66053906892e-24
#define C_MB 1.6737747126723517e-24
#define C_PI 3.14159265358979323846264338328
#define C_H 4.135667696e-21
#define C_HBAR (0.5 * C_H / C_PI)
#define C_CLIGHT 2.99792458e+17
#define C_GF0 1.1663787e-11
#define C_GF (C_GF0 * CUBE(C_HBAR * C_CLIGHT))
#define C_SAT_N 0.15e+18

/* constants.hpp:97-106: couplings and neutral-current form factors */
#define C_GA 1.23
#define C_GV 1.
#define C_GS 0.
#define C_SINTHW2 0.2325
#define C_HNV (-0.5)
#define C_HNA (-0.5 * C_GA)
#define C_HPV (0.5 - 2. * C_SINTHW2)
#define C_HPA (0.5 * C_GA)

/* constants.hpp:109-111 */
#define C_BETA_CONST \
    ((CUBE(C_CLIGHT) * SQ(C_GF0 * C_HBAR)) * (SQ(C_GV) + 3. * SQ(C_GA)) / C_PI)

/* constants.hpp:121-138 */
#define C_ISO_EF (4.785390000313652 * SQ(C_HBAR) / C_MB * C_MEV)
#define C_ISO_CONST (2. * C_PI * SQ(C_GF) / C_HBAR / CUBE(C_H * C_CLIGHT))
#define C_ISO_H0P (SQ(C_HPV) + 3. * SQ(C_HPA))
#define C_ISO_H1P (SQ(C_HPV) - SQ(C_HPA))
#define C_ISO_H0N (SQ(C_HNV) + 3. * SQ(C_HNA))
#define C_ISO_H1N (SQ(C_HNV) - SQ(C_HNA))
#define C_ISO_C0P (C_ISO_CONST * C_ISO_H0P)
#define C_ISO_C1P (C_ISO_CONST * C_ISO_H1P)
#define C_ISO_C0N (C_ISO_CONST * C_ISO_H0N)
#define C_ISO_C1N (C_ISO_CONST * C_ISO_H1N)

/* constants.hpp:145-159 */
#define C_BREM_XMIN 1.0e-10
#define C_BREM_YMIN 1.0e-10
#define C_BREM_ETAMIN 1.0e-10
#define C_BREM_AUX1 (0.25 * SQ(C_H) * C_MEV / SQ(C_PI))
#define C_BREM_CA (-0.63)
#define C_BREM_CONST (SQ(C_BREM_CA) * SQ(C_GF) / C_HBAR)
#define C_BREM_C4BRT06 0.1409912109375

/* constants.hpp:167-183 */
#define C_PAIR_PHI (1.55e-12 / C_PI)
#define C_PAIR_A1E (1. + 2. * C_SINTHW2)
#define C_PAIR_A2E (2. * C_SINTHW2)
#define C_PAIR_A1X (-1. + 2. * C_SINTHW2)
#define C_PAIR_A2X (2. * C_SINTHW2)

/* constants.hpp:190-196 */
#define C_NEPS_CONST \
    (2. * SQ(C_GF0) * C_CLIGHT * SQ(C_HBAR * C_CLIGHT) / (3. * C_PI))
#define C_NEPS_BPLUS SQ(2. * C_SINTHW2 + 1.)
#define C_NEPS_BMINUS SQ(2. * C_SINTHW2 - 1.)
#define C_NEPS_BZERO (4. * SQ(C_SINTHW2))

/* constants.hpp:204-244 */
#define C_EXP_UPP 700.
#define C_EXP_LOW (-700.)
#define C_HC6_4PI2 \
    ((C_H * C_CLIGHT) * (C_H * C_CLIGHT) * (C_H * C_CLIGHT) * (C_H * C_CLIGHT) * \
     (C_H * C_CLIGHT) * (C_H * C_CLIGHT) / (16. * SQ(C_PI)))
#define C_WM_ESCALE (C_MEV / (C_MB * SQ(C_CLIGHT)))
#define C_FOURPI_HC3 ((4. * C_PI) / CUBE(C_H * C_CLIGHT))
#define C_FOURPI_HC3_SQR SQ(C_FOURPI_HC3)
#define C_MN_GRAMS (C_MN * C_MEV / SQ(C_CLIGHT))
#define C_MP_GRAMS (C_MP * C_MEV / SQ(C_CLIGHT))
#define C_MAVG_GRAMS (C_MEV / SQ(C_CLIGHT) * 938.918532994116257276238085018813)
#define C_SQRTPI 1.77245385090551602729816748334106
#define C_PISQ 9.86960440108935861883449099987572
#define C_FOURPISQ 39.4784176043574344753379639995029
#define C_PI_1_8 1.15383506784998943054096521314981
#define C_PIHALF_5_2 3.09242868139914350627854469835251

/* functions.hpp:22 */
#define C_FDI_LIT 7.38905609893065023

#endif

/* IMEX Runge-Kutta Butcher tableaux of src/timeschemes.F90 (implicit tables
 * :1055-1610, explicit tables :1700-2390, constants :186-1000), with the
 * reference's per-scheme flags: ars_eqn_check_D / _A (stiffly accurate
 * implicit / explicit part: the last row of a equals b, set by hand or by
 * comparing the last row for some schemes), diag_diff (the diagonal of the
 * implicit table varies by stage) and diag_index (the stage, 1-based, whose
 * diagonal entry builds the implicit operators).  The coefficients are the
 * published ones; they are written here with the same expressions so that
 * they round to the same doubles.  Shared by the GPU host and the CPU
 * oracle (C and C++). */
#ifndef FALCON_IMEXRK_TABLES_H
#define FALCON_IMEXRK_TABLES_H

#include <math.h>
#include <string.h>

#define IMEXRK_MAX_STAGES 8

/* Scheme numbers (time_scheme_imp / time_scheme_exp; the explicit partner
 * "expXXX" has the same number). */
enum {
  IMEXRK_ARS443 = 10, IMEXRK_ARS343 = 11, IMEXRK_BPR353 = 12, IMEXRK_ARS222 = 13,
  IMEXRK_ARS232 = 14, IMEXRK_ARS233 = 15,
  IMEXRK_EUL111 = 30, IMEXRK_MARS343 = 31, IMEXRK_IJ3 = 32, IMEXRK_PC2 = 33, IMEXRK_SSP332 = 34,
  IMEXRK_SSP543 = 35, IMEXRK_PR433 = 36, IMEXRK_DBM453 = 37, IMEXRK_KC343 = 38, IMEXRK_KC564 = 39,
  IMEXRK_FW53 = 40, IMEXRK_CK222 = 41, IMEXRK_BPR442 = 42, IMEXRK_CFN343 = 43, IMEXRK_BHR553 = 44,
  IMEXRK_CFN564 = 45,
  /* recognised, not built: stage-dependent implicit diagonal (diag_diff) or more than 6 stages */
  IMEXRK_KC774 = 46, IMEXRK_KC885 = 47, IMEXRK_SMR333 = 48, IMEXRK_CB3E = 49, IMEXRK_CB3F = 50,
  IMEXRK_CB4 = 51, IMEXRK_LZ3L1 = 52, IMEXRK_LZ3A4A = 53, IMEXRK_LZ4A1 = 54
};

typedef struct {
  int n;                                   /* stages */
  double aD[IMEXRK_MAX_STAGES][IMEXRK_MAX_STAGES], bD[IMEXRK_MAX_STAGES];
  double aA[IMEXRK_MAX_STAGES][IMEXRK_MAX_STAGES], bA[IMEXRK_MAX_STAGES];
  int check_D, check_A;                    /* ars_eqn_check_D / _A */
  int diag_diff, diag_index;               /* diag_index is 1-based */
} imexrk_table;

static inline void imexrk_fill_(imexrk_table* t, int n, const double* aD, const double* bD, const double* aA,
                                const double* bA) {
  int i, j;
  t->n = n;
  for (i = 0; i < n; ++i) {
    for (j = 0; j < n; ++j) { t->aD[i][j] = aD[i * n + j]; t->aA[i][j] = aA[i * n + j]; }
    t->bD[i] = bD[i]; t->bA[i] = bA[i];
  }
}

/* ars_eqn_check by comparison: true if any last-row entry equals b */
static inline int imexrk_last_row_match_(int n, const double a[IMEXRK_MAX_STAGES][IMEXRK_MAX_STAGES],
                                         const double* b) {
  int i, m = 0;
  for (i = 0; i < n; ++i)
    if (a[n - 1][i] == b[i]) m = 1;
  return m;
}

/* Fills t for the pair (imp, exp); returns 0, or -1 when the pair is not
 * a matching implicit/explicit couple or is not built (see above). */
static inline int imexrk_table_get(int imp, int exp, imexrk_table* t) {
  memset(t, 0, sizeof(*t));
  t->diag_index = 2;
  if (imp != exp) return -1;
  switch (imp) {
    case IMEXRK_ARS443: {
      const double aD[25] = {0, 0, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1.0 / 6.0, 0.5, 0, 0,
                             0, -0.5, 0.5, 0.5, 0, 0, 1.5, -1.5, 0.5, 0.5};
      const double bD[5] = {0, 1.5, -1.5, 0.5, 0.5};
      const double aA[25] = {0, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 11.0 / 18.0, 1.0 / 18.0, 0, 0, 0,
                             5.0 / 6.0, -5.0 / 6.0, 0.5, 0, 0, 0.25, 7.0 / 4.0, 0.75, -7.0 / 4.0, 0};
      const double bA[5] = {0.25, 7.0 / 4.0, 0.75, -7.0 / 4.0, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = imexrk_last_row_match_(5, t->aD, t->bD);
      t->check_A = imexrk_last_row_match_(5, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_BPR353: {
      const double aD[25] = {0, 0, 0, 0, 0, 0.5, 0.5, 0, 0, 0, 5.0 / 18.0, -1.0 / 9.0, 0.5, 0, 0,
                             0.5, 0, 0, 0.5, 0, 0.25, 0, 0.75, -0.5, 0.5};
      const double bD[5] = {0.25, 0, 0.75, -0.5, 0.5};
      const double aA[25] = {0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 4.0 / 9.0, 2.0 / 9.0, 0, 0, 0,
                             0.25, 0, 0.75, 0, 0, 0.25, 0, 0.75, 0, 0};
      const double bA[5] = {0.25, 0, 0.75, 0, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = imexrk_last_row_match_(5, t->aD, t->bD);
      t->check_A = imexrk_last_row_match_(5, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_ARS343: {
      const double g = 0.435866521508459;
      const double bb1 = -1.5 * g * g + 4.0 * g - 0.25, bb2 = 1.5 * g * g - 5.0 * g + 1.25;
      const double aD[16] = {0, 0, 0, 0, 0, g, 0, 0, 0, 0.5 * (1.0 - g), g, 0, 0, bb1, bb2, g};
      const double bD[4] = {0, bb1, bb2, g};
      const double aA[16] = {0, 0, 0, 0, g, 0, 0, 0, 0.3212788860286278, 0.3966543747256017, 0, 0,
                             -0.1058582960718797, 0.5529291480359398, 0.5529291480359398, 0};
      const double bA[4] = {0, bb1, bb2, g};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_ARS222: {
      const double g = (2.0 - sqrt(2.0)) / 2.0, dl = 1.0 - 1.0 / g / 2.0;
      const double aD[9] = {0, 0, 0, 0, g, 0, 0, 1.0 - g, g};
      const double bD[3] = {0, 1.0 - g, g};
      const double aA[9] = {0, 0, 0, g, 0, 0, dl, 1.0 - dl, 0};
      const double bA[3] = {dl, 1.0 - dl, 0};
      imexrk_fill_(t, 3, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1;
      return 0;
    }
    case IMEXRK_ARS232: {
      const double g = (2.0 - sqrt(2.0)) / 2.0, dl = -2.0 * sqrt(2.0) / 3.0;
      const double aD[9] = {0, 0, 0, 0, g, 0, 0, 1.0 - g, g};
      const double bD[3] = {0, 1.0 - g, g};
      const double aA[9] = {0, 0, 0, g, 0, 0, dl, 1.0 - dl, 0};
      const double bA[3] = {0, 1.0 - g, g};
      imexrk_fill_(t, 3, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_ARS233: {
      const double g = (3.0 + sqrt(3.0)) / 6.0;
      const double aD[9] = {0, 0, 0, 0, g, 0, 0, 1.0 - 2.0 * g, g};
      const double bD[3] = {0, 0.5, 0.5};
      const double aA[9] = {0, 0, 0, g, 0, 0, g - 1.0, 2.0 * (1.0 - g), 0};
      const double bA[3] = {0, 0.5, 0.5};
      imexrk_fill_(t, 3, aD, bD, aA, bA);
      t->check_D = 0; t->check_A = 0;
      return 0;
    }
    case IMEXRK_EUL111: {
      const double aD[4] = {0, 0, 0, 1.0};
      const double bD[2] = {0, 1.0};
      const double aA[4] = {0, 0, 1.0, 0};
      const double bA[2] = {1.0, 0};
      imexrk_fill_(t, 2, aD, bD, aA, bA);
      t->check_D = 0; t->check_A = 0;  /* neither is set by the reference */
      return 0;
    }
    case IMEXRK_MARS343: {
      const double g = 0.435866521508458;
      const double aD[16] = {0, 0, 0, 0, 0, g, 0, 0, 0, 0.28206673924577, g, 0,
                             0, 1.20849664917601, -0.64436317068446, g};
      const double bD[4] = {0, 1.20849664917601, -0.64436317068446, g};
      const double aA[16] = {0, 0, 0, 0, g, 0, 0, 0, 0.535396540307354, 0.182536720446875, 0, 0,
                             0.63041255815287, -0.83193390106308, 1.20152134291021, 0};
      const double bA[4] = {0, 1.20849664917601, -0.64436317068446, g};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_IJ3: {
      const double l = 0.7886866510998523;
      const double aD[16] = {0, 0, 0, 0,
                             0, l, 0, 0,
                             0, l / (3.0 * (1.0 - 2.0 * l)), (1.0 - 3.0 * l) / (3.0 * (1.0 - 2.0 * l)), 0,
                             0, -1.0 * l / (1.0 - 2.0 * l), (1.0 - l) / (1.0 - 2.0 * l), 0};
      const double bD[4] = {0, 0, 0.75, 0.25};
      const double aA[16] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 1.0 / 3.0, 0, 0, 0, -1.0, 2.0, 0};
      const double bA[4] = {0, 0, 0.75, 0.25};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 0; t->check_A = 0;
      return 0;
    }
    case IMEXRK_PC2: {
      const double aD[16] = {0, 0, 0, 0, 0.5, 0.5, 0, 0, 0.5, 0, 0.5, 0, 0.5, 0, 0, 0.5};
      const double bD[4] = {0.5, 0, 0, 0.5};
      const double aA[16] = {0, 0, 0, 0, 1.0, 0, 0, 0, 0.5, 0.5, 0, 0, 0.5, 0, 0.5, 0};
      const double bA[4] = {0.5, 0, 0.5, 0};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1;
      return 0;
    }
    case IMEXRK_SSP332: {
      const double aD[16] = {0, 0, 0, 0, 0, 0.5, 0, 0, 0, 0.5, 0.5, 0, 0, 1.0, -0.5, 0.5};
      const double bD[4] = {0, 1.0, -0.5, 0.5};
      const double aA[16] = {0, 0, 0, 0, 0.5, 0, 0, 0, 0.5, 0.5, 0, 0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0};
      const double bA[4] = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1;
      return 0;
    }
    case IMEXRK_SSP543: {
      const double aD[36] = {0, 0, 0, 0, 0, 0,
                             0, 0.5, 0, 0, 0, 0,
                             0, 0.5, 0.5, 0, 0, 0,
                             0, 0.5, -0.5, 0.5, 0, 0,
                             0, 2.0, 0.5, -3.0, 0.5, 0,
                             0, 2.0 / 3.0, -1.0 / 3.0, 0, 1.0 / 6.0, 0.5};
      const double bD[6] = {0, 2.0 / 3.0, -1.0 / 3.0, 0, 1.0 / 6.0, 0.5};
      const double aA[36] = {0, 0, 0, 0, 0, 0,
                             0.5, 0, 0, 0, 0, 0,
                             0.5, 0.5, 0, 0, 0, 0,
                             1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 0, 0, 0,
                             0, 0, 0, 0, 0, 0,
                             1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 0.5, 0, 0};
      const double bA[6] = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 0.5, 0, 0};
      imexrk_fill_(t, 6, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1;
      return 0;
    }
    case IMEXRK_PR433: {
      const double al = 0.24169426078821, be = 0.06042356519705, et = 0.12915286960590;
      const double aD[25] = {0, 0, 0, 0, 0,
                             0, al, 0, 0, 0,
                             0, -al, al, 0, 0,
                             0, 0, 1.0 - al, al, 0,
                             0, be, et, 0.5 - be - et - al, al};
      const double bD[5] = {0, 0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
      const double aA[25] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 0.25, 0.25, 0};
      const double bA[5] = {0, 0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 0; t->check_A = 0;
      return 0;
    }
    case IMEXRK_DBM453: {
      const double aD[25] = {0, 0, 0, 0, 0,
                             -0.22284985318525410, 0.32591194130117247, 0, 0, 0,
                             -0.46801347074080545, 0.86349284225716961, 0.32591194130117247, 0, 0,
                             -0.46509906651927421, 0.81063103116959553, 0.61036726756832357, 0.32591194130117247, 0,
                             0.87795339639076675, -0.72692641526151547, 0.75204137157372720, -0.22898029400415088,
                             0.32591194130117247};
      const double bD[5] = {0.87795339639076672, -0.72692641526151549, 0.7520413715737272, -0.22898029400415090,
                            0.32591194130117247};
      const double aA[25] = {0, 0, 0, 0, 0,
                             0.10306208811591838, 0, 0, 0, 0,
                             -0.94124866143519894, 1.6626399742527356, 0, 0, 0,
                             -1.3670975201437765, 1.3815852911016873, 1.2673234025619065, 0, 0,
                             -0.81287582068772448, 0.81223739060505738, 0.90644429603699305, 0.094194134045674111, 0};
      const double bA[5] = {0.87795339639076672, -0.72692641526151549, 0.7520413715737272, -0.22898029400415090,
                            0.32591194130117247};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_KC343: {
      const double g = 1767732205903.0 / 4055673282236.0;
      const double b1 = 1471266399579.0 / 7840856788654.0, b2 = -4482444167858.0 / 7529755066697.0;
      const double b3 = 11266239266428.0 / 11593286722821.0;
      const double aD[16] = {0, 0, 0, 0,
                             g, g, 0, 0,
                             2746238789719.0 / 10658868560708.0, -640167445237.0 / 6845629431997.0, g, 0,
                             b1, b2, b3, g};
      const double bD[4] = {b1, b2, b3, g};
      const double aA[16] = {0, 0, 0, 0,
                             1767732205903.0 / 2027836641118.0, 0, 0, 0,
                             5535828885825.0 / 10492691773637.0, 788022342437.0 / 10882634858940.0, 0, 0,
                             6485989280629.0 / 16251701735622.0, -4246266847089.0 / 9704473918619.0,
                             10755448449292.0 / 10357097424841.0, 0};
      const double bA[4] = {b1, b2, b3, g};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = imexrk_last_row_match_(4, t->aD, t->bD);
      t->check_A = imexrk_last_row_match_(4, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_KC564: {
      const double b1 = 82889.0 / 524892.0, b3 = 15625.0 / 83664.0, b4 = 69875.0 / 102672.0, b5 = -2260.0 / 8211.0;
      const double aD[36] = {0, 0, 0, 0, 0, 0,
                             0.25, 0.25, 0, 0, 0, 0,
                             8611.0 / 62500.0, -1743.0 / 31250.0, 0.25, 0, 0, 0,
                             5012029.0 / 34652500.0, -654441.0 / 2922500.0, 174375.0 / 388108.0, 0.25, 0, 0,
                             15267082809.0 / 155376265600.0, -71443401.0 / 120774400.0, 730878875.0 / 902184768.0,
                             2285395.0 / 8070912.0, 0.25, 0,
                             b1, 0, b3, b4, b5, 0.25};
      const double bD[6] = {b1, 0, b3, b4, b5, 0.25};
      const double aA[36] = {0, 0, 0, 0, 0, 0,
                             0.5, 0, 0, 0, 0, 0,
                             13861.0 / 62500.0, 6889.0 / 62500.0, 0, 0, 0, 0,
                             -116923316275.0 / 2393684061468.0, -2731218467317.0 / 15368042101831.0,
                             9408046702089.0 / 11113171139209.0, 0, 0, 0,
                             -451086348788.0 / 2902428689909.0, -2682348792572.0 / 7519795681897.0,
                             12662868775082.0 / 11960479115383.0, 3355817975965.0 / 11060851509271.0, 0, 0,
                             647845179188.0 / 3216320057751.0, 73281519250.0 / 8382639484533.0,
                             552539513391.0 / 3454668386233.0, 3354512671639.0 / 8306763924573.0, 4040.0 / 17871.0, 0};
      const double bA[6] = {b1, 0, b3, b4, b5, 0.25};
      imexrk_fill_(t, 6, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_FW53: {
      const double aD[25] = {0, 0, 0, 0, 0,
                             0, 1.0, 0, 0, 0,
                             0.5, 0, 0.5, 0, 0,
                             0.25, -0.25, 0, 0.5, 0,
                             1.0 / 6.0, 1.0 / 6.0, -1.0 / 6.0, 4.0 / 6.0, 1.0 / 6.0};
      const double bD[5] = {1.0 / 6.0, 1.0 / 6.0, -1.0 / 6.0, 4.0 / 6.0, 1.0 / 6.0};
      const double aA[25] = {0, 0, 0, 0, 0,
                             1.0, 0, 0, 0, 0,
                             0.5, 0.5, 0, 0, 0,
                             0.25, 0.25, 0, 0, 0,
                             1.0 / 6.0, 1.0 / 6.0, 0, 4.0 / 6.0, 0};
      const double bA[5] = {1.0 / 6.0, 1.0 / 6.0, 0, 4.0 / 6.0, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = imexrk_last_row_match_(5, t->aD, t->bD);
      t->check_A = imexrk_last_row_match_(5, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_CK222: {
      const double s2 = sqrt(2.0), third = 1.0 / 3.0, tq = 3.0 / 4.0;
      const double aD[9] = {0, 0, 0,
                            -third + s2 * 0.5, 1.0 - s2 * 0.5, 0,
                            tq - s2 * 0.25, -tq + s2 * 0.75, 1.0 - s2 * 0.5};
      const double bD[3] = {tq - s2 * 0.25, -tq + s2 * 0.75, 1.0 - s2 * 0.5};
      const double aA[9] = {0, 0, 0, 2.0 / 3.0, 0, 0, 0.25, 0.75, 0};
      const double bA[3] = {0.25, 0.75, 0};
      imexrk_fill_(t, 3, aD, bD, aA, bA);
      t->check_D = imexrk_last_row_match_(3, t->aD, t->bD);
      t->check_A = imexrk_last_row_match_(3, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_BPR442: {
      const double aD[25] = {0, 0, 0, 0, 0,
                             0, 0.25, 0, 0, 0,
                             0, 0, 0.25, 0, 0,
                             0, 1.0 / 24.0, 11.0 / 24.0, 0.25, 0,
                             0, 11.0 / 24.0, 1.0 / 6.0, 1.0 / 8.0, 0.25};
      const double bD[5] = {0, 11.0 / 24.0, 1.0 / 6.0, 1.0 / 8.0, 0.25};
      const double aA[25] = {0, 0, 0, 0, 0,
                             0.25, 0, 0, 0, 0,
                             13.0 / 4.0, -3.0, 0, 0, 0,
                             0.25, 0, 0.5, 0, 0,
                             0, 1.0 / 3.0, 1.0 / 6.0, 0.5, 0};
      const double bA[5] = {0, 1.0 / 3.0, 1.0 / 6.0, 0.5, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 1;
      t->check_A = imexrk_last_row_match_(5, t->aA, t->bA);
      return 0;
    }
    case IMEXRK_CFN343: {
      const double g = 0.435866521508459;
      const double aD[16] = {0, 0, 0, 0,
                             0, g, 0, 0,
                             0, (1.0 - g) / 2.0, g, 0,
                             0, 1.208496649176010, -0.644363170684469, g};
      const double bD[4] = {0, 1.208496649176010, -0.644363170684469, g};
      const double aA[16] = {0, 0, 0, 0,
                             g, 0, 0, 0,
                             (1.0 + g) / 2.0 + 0.35, -0.35, 0, 0,
                             0, 1.0 + 0.989175724679846, -0.989175724679846, 0};
      const double bA[4] = {0, 1.208496649176010, -0.644363170684469, g};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_BHR553: {
      const double g = 0.435866521508482;
      const double aa31 = g, aa32 = aa31;
      const double aa41 = -475883375220285986033264.0 / 594112726933437845704163.0, aa42 = 0.0;
      const double aa43 = 1866233449822026827708736.0 / 594112726933437845704163.0;
      const double aa51 = 62828845818073169585635881686091391737610308247.0 /
                          176112910684412105319781630311686343715753056000.0;
      const double aa52 = -302987763081184622639300143137943089.0 / 1535359944203293318639180129368156500.0;
      const double aa53 = 262315887293043739337088563996093207.0 / 297427554730376353252081786906492000.0;
      const double aa54 = -987618231894176581438124717087.0 / 23877337660202969319526901856000.0;
      const double a31 = aa31;
      const double a32 = -31733082319927313.0 / 455705377221960889379854647102.0;
      const double a41 = -3012378541084922027361996761794919360516301377809610.0 /
                         45123394056585269977907753045030512597955897345819349.0;
      const double a42 = -62865589297807153294268.0 / 102559673441610672305587327019095047.0;
      const double a43 = 418769796920855299603146267001414900945214277000.0 /
                         212454360385257708555954598099874818603217167139.0;
      const double bb1 = 487698502336740678603511.0 / 1181159636928185920260208.0;
      const double bb3 = -1.0 * aa52;
      const double bb4 = -105235928335100616072938218863.0 / 2282554452064661756575727198000.0;
      const double aD[25] = {0, 0, 0, 0, 0,
                             g, g, 0, 0, 0,
                             a31, a32, g, 0, 0,
                             a41, a42, a43, g, 0,
                             bb1, 0, bb3, bb4, g};
      const double bD[5] = {bb1, 0, bb3, bb4, g};
      const double aA[25] = {0, 0, 0, 0, 0,
                             2.0 * g, 0, 0, 0, 0,
                             aa31, aa32, 0, 0, 0,
                             aa41, aa42, aa43, 0, 0,
                             aa51, aa52, aa53, aa54, 0};
      const double bA[5] = {bb1, 0, bb3, bb4, g};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_CFN564: {
      const double b[6] = {0, 25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25};
      const double aD[36] = {0, 0, 0, 0, 0, 0,
                             0, 0.25, 0, 0, 0, 0,
                             0, 0.5, 0.25, 0, 0, 0,
                             0, 17.0 / 50.0, -1.0 / 25.0, 0.25, 0, 0,
                             0, 371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0, 0.25, 0,
                             b[0], b[1], b[2], b[3], b[4], b[5]};
      const double aA[36] = {0, 0, 0, 0, 0, 0,
                             0.25, 0, 0, 0, 0, 0,
                             -0.25, 1.0, 0, 0, 0, 0,
                             -13.0 / 100.0, 43.0 / 75.0, 8.0 / 75.0, 0, 0, 0,
                             -6.0 / 85.0, 42.0 / 85.0, 179.0 / 1360.0, -15.0 / 272.0, 0, 0,
                             0, 79.0 / 24.0, -5.0 / 8.0, 25.0 / 2.0, -85.0 / 6.0, 0};
      imexrk_fill_(t, 6, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    default:
      return -1;
  }
}

/* Scheme name (without the "exp" prefix of the explicit partner) -> number,
 * or -1. */
static inline int imexrk_scheme_id(const char* name) {
  static const struct { const char* n; int id; } k[] = {
      {"ARS443", IMEXRK_ARS443}, {"ARS343", IMEXRK_ARS343}, {"BPR353", IMEXRK_BPR353}, {"ARS222", IMEXRK_ARS222},
      {"ARS232", IMEXRK_ARS232}, {"ARS233", IMEXRK_ARS233}, {"EUL111", IMEXRK_EUL111}, {"MARS343", IMEXRK_MARS343},
      {"IJ3", IMEXRK_IJ3}, {"PC2", IMEXRK_PC2}, {"SSP332", IMEXRK_SSP332}, {"SSP543", IMEXRK_SSP543},
      {"PR433", IMEXRK_PR433}, {"DBM453", IMEXRK_DBM453}, {"KC343", IMEXRK_KC343}, {"KC564", IMEXRK_KC564},
      {"FW53", IMEXRK_FW53}, {"CK222", IMEXRK_CK222}, {"BPR442", IMEXRK_BPR442}, {"CFN343", IMEXRK_CFN343},
      {"BHR553", IMEXRK_BHR553}, {"CFN564", IMEXRK_CFN564}, {"KC774", IMEXRK_KC774}, {"KC885", IMEXRK_KC885},
      {"SMR333", IMEXRK_SMR333}, {"CB3E", IMEXRK_CB3E}, {"CB3F", IMEXRK_CB3F}, {"CB4", IMEXRK_CB4},
      {"LZ3L1", IMEXRK_LZ3L1}, {"LZ3A4A", IMEXRK_LZ3A4A}, {"LZ4A1", IMEXRK_LZ4A1}};
  for (unsigned i = 0; i < sizeof(k) / sizeof(k[0]); ++i)
    if (strcmp(name, k[i].n) == 0) return k[i].id;
  return -1;
}

#endif

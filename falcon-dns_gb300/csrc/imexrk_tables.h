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
  /* 7 and 8 stages */
  IMEXRK_KC774 = 46, IMEXRK_KC885 = 47,
  /* stage-dependent implicit diagonal (diag_diff) */
  IMEXRK_SMR333 = 48, IMEXRK_CB3E = 49, IMEXRK_CB3F = 50,
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
 * a matching implicit/explicit couple. */
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
    case IMEXRK_KC774: {
      /* ESDIRK: every implicit stage after the first has the diagonal 0.1235 */
      const double g = 0.1235;
      const double a21 = 624185399699.0 / 4186980696204.0, a31 = 1258591069120.0 / 10082082980243.0;
      const double a33 = -322722984531.0 / 8455138723562.0, a41 = -436103496990.0 / 5971407786587.0;
      const double a43 = -2689175662187.0 / 11046760208243.0, a44 = 4431412449334.0 / 12995360898505.0;
      const double a51 = -2207373168298.0 / 14430576638973.0, a53 = 242511121179.0 / 3358618340039.0;
      const double a54 = 3145666661981.0 / 7780404714551.0, a55 = 5882073923981.0 / 14490790706663.0;
      const double b3 = 9164257142617.0 / 17756377923965.0, b4 = -10812980402763.0 / 74029279521829.0;
      const double b5 = 1335994250573.0 / 5691609445217.0, b6 = 2273837961795.0 / 8368240463276.0;
      const double aD[49] = {0, 0, 0, 0, 0, 0, 0,
                             g, g, 0, 0, 0, 0, 0,
                             a21, a21, g, 0, 0, 0, 0,
                             a31, a31, a33, g, 0, 0, 0,
                             a41, a41, a43, a44, g, 0, 0,
                             a51, a51, a53, a54, a55, g, 0,
                             0, 0, b3, b4, b5, b6, g};
      const double b[7] = {0, 0, b3, b4, b5, b6, g};
      const double e61 = 760814592956.0 / 3276306540349.0;
      const double aA[49] = {0, 0, 0, 0, 0, 0, 0,
                             0.247, 0, 0, 0, 0, 0, 0,
                             0.06175, 2694949928731.0 / 7487940209513.0, 0, 0, 0, 0, 0,
                             464650059369.0 / 8764239774964.0, 878889893998.0 / 2444806327765.0,
                             -952945855348.0 / 12294611323341.0, 0, 0, 0, 0,
                             476636172619.0 / 8159180917465.0, -1271469283451.0 / 7793814740893.0,
                             -859560642026.0 / 4356155882851.0, 1723805262919.0 / 4571918432560.0, 0, 0, 0,
                             6338158500785.0 / 11769362343261.0, -4970555480458.0 / 10924838743837.0,
                             3326578051521.0 / 2647936831840.0, -880713585975.0 / 1841400956686.0,
                             -1428733748635.0 / 8843423958496.0, 0, 0,
                             e61, e61, -47223648122716.0 / 6934462133451.0, 71187472546993.0 / 9669769126921.0,
                             -13330509492149.0 / 9695768672337.0, 11565764226357.0 / 8513123442827.0, 0};
      imexrk_fill_(t, 7, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    case IMEXRK_KC885: {
      const double g = 2.0 / 9.0;
      const double a21 = 2366667076620.0 / 8822750406821.0, a31 = -257962897183.0 / 4451812247028.0;
      const double a33 = 128530224461.0 / 14379561246022.0, a41 = -486229321650.0 / 11227943450093.0;
      const double a43 = -225633144460.0 / 6633558740617.0, a44 = 1741320951451.0 / 6824444397158.0;
      const double a51 = 621307788657.0 / 4714163060173.0, a53 = -125196015625.0 / 3866852212004.0;
      const double a54 = 940440206406.0 / 7593089888465.0, a55 = 961109811699.0 / 6734810228204.0;
      const double a61 = 2036305566805.0 / 6583108094622.0, a63 = -3039402635899.0 / 4450598839912.0;
      const double a64 = -1829510709469.0 / 31102090912115.0, a65 = -286320471013.0 / 6931253422520.0;
      const double a66 = 8651533662697.0 / 9642993110008.0;
      const double b3 = 3517720773327.0 / 20256071687669.0, b4 = 4569610470461.0 / 17934693873752.0;
      const double b5 = 2819471173109.0 / 11655438449929.0, b6 = 3296210113763.0 / 10722700128969.0;
      const double b7 = -1142099968913.0 / 5710983926999.0;
      const double aD[64] = {0, 0, 0, 0, 0, 0, 0, 0,
                             g, g, 0, 0, 0, 0, 0, 0,
                             a21, a21, g, 0, 0, 0, 0, 0,
                             a31, a31, a33, g, 0, 0, 0, 0,
                             a41, a41, a43, a44, g, 0, 0, 0,
                             a51, a51, a53, a54, a55, g, 0, 0,
                             a61, a61, a63, a64, a65, a66, g, 0,
                             0, 0, b3, b4, b5, b6, b7, g};
      const double b[8] = {0, 0, b3, b4, b5, b6, b7, g};
      const double e71 = 2193717860234.0 / 3570523412979.0;
      const double aA[64] = {0, 0, 0, 0, 0, 0, 0, 0,
                             4.0 / 9.0, 0, 0, 0, 0, 0, 0, 0,
                             1.0 / 9.0, 1183333538310.0 / 1827251437969.0, 0, 0, 0, 0, 0, 0,
                             895379019517.0 / 9750411845327.0, 477606656805.0 / 13473228687314.0,
                             -112564739183.0 / 9373365219272.0, 0, 0, 0, 0, 0,
                             -4458043123994.0 / 13015289567637.0, -2500665203865.0 / 9342069639922.0,
                             983347055801.0 / 8893519644487.0, 2185051477207.0 / 2551468980502.0, 0, 0, 0, 0,
                             -167316361917.0 / 17121522574472.0, 1605541814917.0 / 7619724128744.0,
                             991021770328.0 / 13052792161721.0, 2342280609577.0 / 11279663441611.0,
                             3012424348531.0 / 12792462456678.0, 0, 0, 0,
                             6680998715867.0 / 14310383562358.0, 5029118570809.0 / 3897454228471.0,
                             2415062538259.0 / 6382199904604.0, -3924368632305.0 / 6964820224454.0,
                             -4331110370267.0 / 15021686902756.0, -3944303808049.0 / 11994238218192.0, 0, 0,
                             e71, e71, 5952760925747.0 / 18750164281544.0, -4412967128996.0 / 6196664114337.0,
                             4151782504231.0 / 36106512998704.0, 572599549169.0 / 6265429158920.0,
                             -457874356192.0 / 11306498036315.0, 0};
      imexrk_fill_(t, 8, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0;
      return 0;
    }
    /* The schemes below have a stage-dependent implicit diagonal
     * (diag_diff): each stage whose diagonal differs from that of stage
     * diag_index solves with operators of its own weight. */
    case IMEXRK_SMR333: {
      const double alpha1 = 29.0 / 96.0, alpha2 = -3.0 / 40.0, alpha3 = 1.0 / 6.0;
      const double beta1 = 37.0 / 160.0, beta2 = 5.0 / 24.0, beta3 = 1.0 / 6.0;
      const double gamma1 = 8.0 / 15.0, gamma2 = 5.0 / 12.0, gamma3 = 3.0 / 4.0;
      const double xeta1 = -17.0 / 60.0, xeta2 = -5.0 / 12.0;
      const double aD[16] = {0, 0, 0, 0,
                             alpha1, beta1, 0, 0,
                             alpha1, alpha2 + beta1, beta2, 0,
                             alpha1, alpha2 + beta1, alpha3 + beta2, beta3};
      const double bD[4] = {alpha1, alpha2 + beta1, alpha3 + beta2, beta3};
      const double aA[16] = {0, 0, 0, 0,
                             gamma1, 0, 0, 0,
                             xeta1 + gamma1, gamma2, 0, 0,
                             xeta1 + gamma1, xeta2 + gamma2, gamma3, 0};
      const double bA[4] = {xeta1 + gamma1, xeta2 + gamma2, gamma3, 0};
      imexrk_fill_(t, 4, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1; t->diag_diff = 1;
      return 0;
    }
    case IMEXRK_CB3E: {
      const double aD[16] = {0, 0, 0, 0,
                             0, 1.0 / 3.0, 0, 0,
                             0, 0.5, 0.5, 0,
                             0, 0.75, -0.25, 0.5};
      const double b[4] = {0, 0.75, -0.25, 0.5};
      const double aA[16] = {0, 0, 0, 0,
                             1.0 / 3.0, 0, 0, 0,
                             0, 1.0, 0, 0,
                             0, 0.75, 0.25, 0};
      imexrk_fill_(t, 4, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0; t->diag_diff = 1; t->diag_index = 3;
      return 0;
    }
    case IMEXRK_CB3F: {
      const double c2 = 49.0 / 50.0;
      const double a21 = c2 / 2.0, a22 = c2 / 2.0;
      const double a31 = -785157464198.0 / 1093480182337.0, a32 = -30736234873.0 / 978681420651.0;
      const double a33 = 983779726483.0 / 1246172347126.0;
      const double bb1 = -2179897048956.0 / 603118880443.0, bb2 = 99189146040.0 / 891495457793.0;
      const double bb3 = 6064140186914.0 / 1415701440113.0, bb4 = 146791865627.0 / 668377518349.0;
      const double aa21 = c2, aa31 = 13244205847.0 / 647648310246.0, aa32 = 13419997131.0 / 686433909488.0;
      const double aa42 = 231677526244.0 / 1085522130027.0, aa43 = 3007879347537.0 / 683461566472.0;
      const double aD[16] = {0, 0, 0, 0,
                             a21, a22, 0, 0,
                             a31, a32, a33, 0,
                             bb1, bb2, bb3, bb4};
      const double b[4] = {bb1, bb2, bb3, bb4};
      const double aA[16] = {0, 0, 0, 0,
                             aa21, 0, 0, 0,
                             aa31, aa32, 0, 0,
                             bb1, aa42, aa43, 0};
      imexrk_fill_(t, 4, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0; t->diag_diff = 1;
      return 0;
    }
    case IMEXRK_CB4: {
      const double c2 = 0.25;
      const double a21 = c2 / 2.0, a22 = c2 / 2.0;
      const double a31 = 216145252607.0 / 961230882893.0, a32 = 257479850128.0 / 1143310606989.0;
      const double a33 = 30481561667.0 / 101628412017.0;
      const double a42 = -381180097479.0 / 1276440792700.0, a43 = -54660926949.0 / 461115766612.0;
      const double a44 = 344309628413.0 / 552073727558.0;
      const double a53 = -100836174740.0 / 861952129159.0, a54 = -250423827953.0 / 1283875864443.0;
      const double a55 = 0.5;
      const double aa21 = c2, aa31 = 153985248130.0 / 1004999853329.0, aa32 = 902825336800.0 / 1512825644809.0;
      const double aa42 = 99316866929.0 / 820744730663.0, aa43 = 82888780751.0 / 969573940619.0;
      const double aa53 = 57501241309.0 / 765040883867.0, aa54 = 76345938311.0 / 676824576433.0;
      const double aa64 = -4099309936455.0 / 6310162971841.0, aa65 = 1395992540491.0 / 933264948679.0;
      const double bb1 = 232049084587.0 / 1377130630063.0, bb2 = 322009889509.0 / 2243393849156.0;
      const double bb3 = -195109672787.0 / 1233165545817.0, bb4 = -340582416761.0 / 705418832319.0;
      const double bb5 = 463396075661.0 / 409972144477.0, bb6 = 323177943294.0 / 1626646580633.0;
      const double aD[36] = {0, 0, 0, 0, 0, 0,
                             a21, a22, 0, 0, 0, 0,
                             a31, a32, a33, 0, 0, 0,
                             bb1, a42, a43, a44, 0, 0,
                             bb1, bb2, a53, a54, a55, 0,
                             bb1, bb2, bb3, bb4, bb5, bb6};
      const double b[6] = {bb1, bb2, bb3, bb4, bb5, bb6};
      const double aA[36] = {0, 0, 0, 0, 0, 0,
                             aa21, 0, 0, 0, 0, 0,
                             aa31, aa32, 0, 0, 0, 0,
                             bb1, aa42, aa43, 0, 0, 0,
                             bb1, bb2, aa53, aa54, 0, 0,
                             bb1, bb2, bb3, aa64, aa65, 0};
      imexrk_fill_(t, 6, aD, b, aA, b);
      t->check_D = 1; t->check_A = 0; t->diag_diff = 1;
      return 0;
    }
    case IMEXRK_LZ3L1: {
      const double aD[25] = {0, 0, 0, 0, 0,
                             3.0 / 20.0, 1.0 / 10.0, 0, 0, 0,
                             9.0 / 10.0, -13.0 / 10.0, 9.0 / 10.0, 0, 0,
                             17.0 / 10.0, -11.0 / 4.0, 3.0 / 2.0, 3.0 / 10.0, 0,
                             1.0, -10.0 / 3.0, 17.0 / 3.0, -10.0 / 3.0, 1.0};
      const double bD[5] = {1.0, -10.0 / 3.0, 17.0 / 3.0, -10.0 / 3.0, 1.0};
      const double aA[25] = {0, 0, 0, 0, 0,
                             0.25, 0, 0, 0, 0,
                             0, 0.5, 0, 0, 0,
                             -0.5, 5.0 / 4.0, 0, 0, 0,
                             0, 2.0 / 3.0, -1.0 / 3.0, 2.0 / 3.0, 0};
      const double bA[5] = {0, 2.0 / 3.0, -1.0 / 3.0, 2.0 / 3.0, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1; t->diag_diff = 1;
      return 0;
    }
    case IMEXRK_LZ3A4A: {
      const double aD[25] = {0, 0, 0, 0, 0,
                             0.5, 0, 0, 0, 0,
                             0.25, -0.75, 1.0, 0, 0,
                             0, -3.0, 4.0, 0, 0,
                             1.0 / 6.0, 0, 2.0 / 3.0, -0.5, 2.0 / 3.0};
      const double bD[5] = {1.0 / 6.0, 0, 2.0 / 3.0, -0.5, 2.0 / 3.0};
      const double aA[25] = {0, 0, 0, 0, 0,
                             0.5, 0, 0, 0, 0,
                             0.25, 0.25, 0, 0, 0,
                             0, 1.0, 0, 0, 0,
                             1.0 / 6.0, 0, 2.0 / 3.0, 1.0 / 6.0, 0};
      const double bA[5] = {1.0 / 6.0, 0, 2.0 / 3.0, 1.0 / 6.0, 0};
      imexrk_fill_(t, 5, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1; t->diag_diff = 1; t->diag_index = 3;
      return 0;
    }
    case IMEXRK_LZ4A1: {
      const double aD[49] = {0, 0, 0, 0, 0, 0, 0,
                             -1.0 / 6.0, 0.5, 0, 0, 0, 0, 0,
                             1.0 / 6.0, -1.0 / 3.0, 0.5, 0, 0, 0, 0,
                             3.0 / 8.0, -3.0 / 8.0, 0, 0.5, 0, 0, 0,
                             1.0 / 8.0, 0, 3.0 / 8.0, -0.5, 0.5, 0, 0,
                             -0.5, 0, 3.0, -2.0, 0, 0.5, 0,
                             1.0 / 6.0, 0, 0, 0, 2.0 / 3.0, -0.5, 2.0 / 3.0};
      const double bD[7] = {1.0 / 6.0, 0, 0, 0, 2.0 / 3.0, -0.5, 2.0 / 3.0};
      const double aA[49] = {0, 0, 0, 0, 0, 0, 0,
                             1.0 / 3.0, 0, 0, 0, 0, 0, 0,
                             1.0 / 6.0, 1.0 / 6.0, 0, 0, 0, 0, 0,
                             1.0 / 8.0, 0, 3.0 / 8.0, 0, 0, 0, 0,
                             1.0 / 8.0, 0, 3.0 / 8.0, 0, 0, 0, 0,
                             0.5, 0, -1.5, 1.0, 1.0, 0, 0,
                             1.0 / 6.0, 0, 0, 0, 2.0 / 3.0, 1.0 / 6.0, 0};
      const double bA[7] = {1.0 / 6.0, 0, 0, 0, 2.0 / 3.0, 1.0 / 6.0, 0};
      imexrk_fill_(t, 7, aD, bD, aA, bA);
      t->check_D = 1; t->check_A = 1; t->diag_diff = 1;
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

/*
 * TEST INFRASTRUCTURE ONLY. Link-time wrappers (-Wl,--wrap=...) around entry
 * points of the unmodified reference STZ code, used to record its event
 * sequence and final state for parity fixtures. Compiled together with the
 * reference's own headers; it changes no reference behaviour.
 *
 * Environment:
 *   STZ_REF_LOG         text log: one 'X step kind site mode' line per
 *                       VoxelShearTransform call (kind 0 thermal, 1 athermal)
 *                       and one 'S step kind time eps0 eps1 eps2 s0 s1 s2' line
 *                       per driver step (kind 0 thermal, 1 athermal, 2 elastic)
 *   STZ_REF_MAX_EVENTS  stop once this many thermal events are done
 *   STZ_REF_MAX_STEPS   stop once this many driver steps are done
 *   STZ_REF_DUMP        binary dump of the final state (fields, then the MRO
 *                       map's types and angles), written at the start of
 *                       the step after the stop condition (i.e. after the
 *                       previous step's print/re-solve), or at Free() when the
 *                       reference stops on its own end condition
 */
#include <stdio.h>
#include <stdlib.h>
#include "bmg.h"
#include "my_fft.h"

void __real_VoxelShearTransform(int mm, int idx);
void __real_KMC(void);
void __real_athermal_plasticity(void);
void __real_ActEnergy(int step);

static FILE* g_log = NULL;
static int g_in = -1;
static long g_max_events = -1, g_max_steps = -1;

static void open_log(void) {
  static int done = 0;
  if (done) return;
  done = 1;
  const char* p = getenv("STZ_REF_LOG");
  if (p) g_log = fopen(p, "w");
  p = getenv("STZ_REF_MAX_EVENTS");
  if (p) g_max_events = atol(p);
  p = getenv("STZ_REF_MAX_STEPS");
  if (p) g_max_steps = atol(p);
}

void __wrap_VoxelShearTransform(int mm, int idx) {
  open_log();
  if (g_log) fprintf(g_log, "X %d %d %d %d\n", step, g_in, idx, mm);
  __real_VoxelShearTransform(mm, idx);
}

static void log_step(int kind) {
  if (!g_log) return;
  fprintf(g_log, "S %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", step, kind, totime,
          EpsAvg[0], EpsAvg[1], EpsAvg[2], Stress[0], Stress[1], Stress[2]);
}

void __wrap_KMC(void) {
  open_log();
  int k0 = kstep;
  g_in = 0;
  __real_KMC();
  g_in = -1;
  log_step(kstep > k0 ? 0 : 2);
}

void __wrap_athermal_plasticity(void) {
  open_log();
  g_in = 1;
  __real_athermal_plasticity();
  g_in = -1;
  log_step(1);
}

static void wr(FILE* f, const void* p, size_t sz, size_t n) { fwrite(p, sz, n, f); }

static int g_dumped = 0;

static void dump_state(long long steps_done) {
  const char* p = getenv("STZ_REF_DUMP");
  if (g_dumped) return;
  g_dumped = 1;
  if (p) {
    FILE* f = fopen(p, "wb");
    long long hdr[5] = {(long long)lsize, steps_done, kstep, astep, estep};
    double sc[7] = {totime, EpsAvg[0], EpsAvg[1], EpsAvg[2], Stress[0], Stress[1], Stress[2]};
    wr(f, hdr, sizeof(long long), 5);
    wr(f, sc, sizeof(double), 7);
    for (int c = 0; c < 3; c++) wr(f, Sigma[c], sizeof(double), (size_t)lsize);
    for (int c = 0; c < 3; c++) wr(f, Eps0[c], sizeof(double), (size_t)lsize);
    for (int m = 0; m < MODES; m++)
      for (int c = 0; c < 3; c++) wr(f, DEps0[m][c], sizeof(double), (size_t)lsize);
    for (int m = 0; m < MODES; m++) wr(f, Q0[m], sizeof(double), (size_t)lsize);
    wr(f, tlast, sizeof(double), (size_t)lsize);
    wr(f, PermSoftening, sizeof(double), (size_t)lsize);
    wr(f, TempSoftening, sizeof(double), (size_t)lsize);
    for (int c = 0; c < 3; c++)
      for (int s = 0; s < lsize; s++) {
        double v = PreDEps0[PreSelectMode[s]][c][s];
        fwrite(&v, sizeof(double), 1, f);
      }
    /* the crystal-like MRO map: types (as doubles) and angles */
    for (int s = 0; s < lsize; s++) {
      double v = (double)MRO[s];
      fwrite(&v, sizeof(double), 1, f);
    }
    wr(f, MROthe0, sizeof(double), (size_t)lsize);
    fclose(f);
  }
  if (g_log) fflush(g_log);
}

void __real_Free(void);
/* normal end of the run (stop condition): dump before the fields are freed */
void __wrap_Free(void) {
  dump_state(step);
  __real_Free();
}

void __wrap_ActEnergy(int st) {
  open_log();
  if ((g_max_events >= 0 && kstep >= g_max_events) || (g_max_steps >= 0 && st - 1 >= g_max_steps))
  {
    dump_state(st - 1);
    if (g_log) fclose(g_log);
    exit(0);
  }
  __real_ActEnergy(st);
}

// falcon_run: the drop-in for the reference's `main input.txt`
// (src/main.F90:14-24 -> solver_init / solver_run / solver_log,
// src/solver.F90:38-132).  It reads the same namelist file, steps one
// annulus instance on the GPU through the C ABI of include/falcon_gpu.h only
// (what a Fortran host would call through ISO_C_BINDING), and writes the
// reference's output files in its formats and at its cadence
// (timeloop_imex / timeloop_imexrk / timeloop_rk, src/steptime*.F90):
//   every n_KE steps      KE_<tag>        dt_new, tot_time, KE, KE_r, KE_phi, KE_upbar  (6ES20.12)
//                         Nusselt_<tag>   tot_time, Nu_top, Nu_bot                      (3ES20.12)
//                         power_<tag>     tot_time, viscous, buoyancy                   (3ES20.12)
//                         upbalance_<tag> Nr lines: radius, d(up_0)/dt, advection, diffusion (4ES20.12)
//                         stdout          dt_new, tot_time, KE
//   every n_KEspec steps  KEspec_<tag>, Temp_spec_<tag>: n_step, m, value      (2I8, ES20.12)
//   every n_checkpoint    checkpoint_%05d (count from n_restart_point)
//   every n_snapshot      snapshot_plot_%05d (count from n_snapshot_point)
// all while tot_time < totaltime; the step that reaches totaltime ends the
// run (no output that step), as does KE > 1e10 (src/output.F90:321-323).
// Files are opened in append mode for each write, like init_output.
//
// Usage: falcon_run <namelist> [--noise SEED AMP]
//   without --noise the initial state is the reference's perturbation
//   (n_init, ampT); with it, the conductive profile plus seeded Gaussian
//   noise of amplitude AMP (the benchmark configurations' initial state).
//   l_restart = .TRUE. restores from checkpoint_<n_restart_point> in the
//   working directory.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/falcon_gpu.h"

namespace {

// Fortran ESw.d edit descriptor: one nonzero leading digit, d decimals, a
// two-digit exponent E+dd (or the three-digit form +ddd without the E),
// right-justified in w characters.
std::string fes(double x, int w = 20, int d = 12) {
  char buf[64];
  if (std::isnan(x)) {
    std::snprintf(buf, sizeof buf, "%*s", w, "NaN");
    return buf;
  }
  if (std::isinf(x)) {
    std::snprintf(buf, sizeof buf, "%*s", w, x < 0 ? "-Infinity" : "Infinity");
    return buf;
  }
  std::snprintf(buf, sizeof buf, "%.*E", d, x);
  std::string s(buf);
  const size_t e = s.find('E');
  const int ex = std::atoi(s.c_str() + e + 1);
  if (std::abs(ex) > 99) s = s.substr(0, e) + (ex < 0 ? "-" : "+") + std::to_string(std::abs(ex));
  if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
  return s;
}

std::string i8(long v) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%8ld", v);
  return buf;
}

bool append(const std::string& path, const std::string& text) {
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return false;
  const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  return std::fclose(f) == 0 && ok;
}

[[noreturn]] void die(const char* what, int rc) {
  std::fprintf(stderr, "falcon_run: %s failed (%d): %s\n", what, rc, falcon_last_error());
  std::exit(1);
}

std::string trimmed(const char* s) {
  std::string t(s);
  while (!t.empty() && (t.back() == ' ' || t.back() == '\0')) t.pop_back();
  return t;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <namelist file> [--noise SEED AMP]\n", argv[0]);
    return 2;
  }
  bool noise = false;
  uint64_t seed = 0;
  double amp = 0.0;
  for (int i = 2; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--noise") && i + 2 < argc) {
      noise = true;
      seed = std::strtoull(argv[i + 1], nullptr, 10);
      amp = std::strtod(argv[i + 2], nullptr);
      i += 2;
    } else {
      std::fprintf(stderr, "falcon_run: unknown argument %s\n", argv[i]);
      return 2;
    }
  }
  const auto start = std::chrono::steady_clock::now();
  falcon_params p;
  int rc;
  if ((rc = falcon_params_read_namelist(argv[1], &p))) die("reading the namelist", rc);
  falcon_handle* h = nullptr;
  if ((rc = falcon_create(&p, &h))) die("falcon_create", rc);
  if (p.l_restart) {
    if ((rc = falcon_restart(h, nullptr))) die("falcon_restart", rc);
  } else if (noise) {
    if ((rc = falcon_init_state(h, 1, amp, seed))) die("falcon_init_state", rc);
  } else {
    if ((rc = falcon_init_state(h, 0, p.ampT, 0))) die("falcon_init_state", rc);
  }
  const std::string tag = trimmed(p.tag);
  const int Nr = p.nr_max, M = p.nm_max + 1;
  const long n0 = p.l_restart ? p.n_restart : 0;
  long count_snap = p.n_snapshot_point, count_chkpnt = p.n_restart_point;
  const long cad[4] = {p.n_snapshot, p.n_checkpoint, p.n_KE, p.n_KEspec};
  std::vector<double> ubal((size_t)4 * Nr), kes(M), tsp(M);
  double host_time = 0.0;  // tot_time as the library accumulates it (constant dt)
  {
    double t;
    falcon_time(h, &t, nullptr, nullptr);
    host_time = t;
  }
  long n_step = n0 + 1, steps_taken = 0;
  const long last = (long)p.n_time_steps + n0;
  bool done = false;
  while (n_step <= last && !done) {
    // steps up to the next output event; with a constant dt also up to the
    // first step whose tot_time reaches totaltime (the library adds the
    // same dt in the same order)
    long k = 1;
    if (!p.l_vartimestep) {
      // steps to the next multiple of each cadence, counted from n_step
      long to_event = last - n_step + 1;
      for (long c : cad)
        if (c > 0) {
          const long next = ((n_step + c - 1) / c) * c;  // first multiple >= n_step
          to_event = std::min(to_event, next - n_step + 1);
        }
      double t = host_time;
      k = 0;
      while (k < to_event) {
        t = t + p.dt;
        ++k;
        if (!(t < p.totaltime)) break;
      }
      host_time = t;
    }
    if ((rc = falcon_step(h, (int)k))) die("falcon_step", rc);
    steps_taken += k;
    n_step += k - 1;
    double tot_time = 0.0, dt_new = 0.0;
    falcon_time(h, &tot_time, &dt_new, nullptr);
    host_time = tot_time;
    if (tot_time < p.totaltime) {
      if (p.n_snapshot > 0 && n_step % p.n_snapshot == 0) {
        char name[64];
        std::snprintf(name, sizeof name, "snapshot_plot_%05ld", ++count_snap);
        if ((rc = falcon_store_snapshot(h, name))) die("falcon_store_snapshot", rc);
      }
      if (p.n_checkpoint > 0 && n_step % p.n_checkpoint == 0) {
        std::printf("%s checkpoint save\n", fes(tot_time, 26, 16).c_str());
        char name[64];
        std::snprintf(name, sizeof name, "checkpoint_%05ld", ++count_chkpnt);
        if ((rc = falcon_store_checkpoint(h, name))) die("falcon_store_checkpoint", rc);
      }
      if (p.n_KE > 0 && n_step % p.n_KE == 0) {
        falcon_diag d;
        rc = falcon_diagnostics(h, &d);
        if (rc && rc != FALCON_EBLOWUP) die("falcon_diagnostics", rc);
        if ((rc = falcon_upbalance(h, ubal.data()))) die("falcon_upbalance", rc);
        std::string ub;
        for (int r = 0; r < Nr; ++r)
          ub += fes(ubal[4 * r]) + fes(ubal[4 * r + 1]) + fes(ubal[4 * r + 2]) + fes(ubal[4 * r + 3]) + "\n";
        if (!append("upbalance_" + tag, ub) ||
            !append("KE_" + tag, fes(d.dt) + fes(d.time) + fes(d.ke) + fes(d.ke_r) + fes(d.ke_phi) +
                                     fes(d.ke_upbar) + "\n") ||
            !append("Nusselt_" + tag, fes(d.time) + fes(d.nu_top) + fes(d.nu_bot) + "\n") ||
            !append("power_" + tag, fes(d.time) + fes(d.vis) + fes(d.buo) + "\n")) {
          std::fprintf(stderr, "falcon_run: cannot write the output files\n");
          return 1;
        }
        std::printf("%s%s%s\n", fes(d.dt, 26, 16).c_str(), fes(d.time, 26, 16).c_str(), fes(d.ke, 26, 16).c_str());
        if (d.ke > 1e10) {  // src/output.F90:321-323
          std::fflush(stdout);
          break;
        }
      }
      if (p.n_KEspec > 0 && n_step % p.n_KEspec == 0) {
        if ((rc = falcon_spectra(h, kes.data(), tsp.data()))) die("falcon_spectra", rc);
        std::string a, b;
        for (int m = 0; m < M; ++m) {
          a += i8(n_step) + i8(m) + fes(kes[m]) + "\n";
          b += i8(n_step) + i8(m) + fes(tsp[m]) + "\n";
        }
        if (!append("KEspec_" + tag, a) || !append("Temp_spec_" + tag, b)) {
          std::fprintf(stderr, "falcon_run: cannot write the spectra files\n");
          return 1;
        }
      }
    } else {
      done = true;
    }
    ++n_step;
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
  // solver_log (src/solver.F90:114-132), to standard error like unit 0
  std::fprintf(stderr, " Total time taken = %.6f seconds.\n", secs);
  std::fprintf(stderr, " Time steps taken = %ld, average time per step = %.6e seconds.\n", steps_taken,
               steps_taken ? secs / (double)steps_taken : 0.0);
  falcon_destroy(h);
  return 0;
}

// api.cpp -- the extern "C" boundary of libgbmd (include/gbmd.h) and the host side of the
// plugins: argument parsing with LPMD's Module semantics, the plugin parameter sets, and FP64
// host evaluation of the potential functionals.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <sstream>
#include <string>

#include "../../include/gbmd.h"
#include "engine.h"

#include <cuda_runtime.h>

using namespace gbmd;

namespace {

thread_local std::string g_last_error;

gbmd_status fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

template <class F>
gbmd_status guarded(F&& f) {
  try {
    f();
    g_last_error.clear();
    return GBMD_OK;
  } catch (const Error& e) {
    return fail(e.status, e.what());
  } catch (const std::bad_alloc&) {
    return fail(GBMD_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(GBMD_ERR_RUNTIME, e.what());
  }
}

double num(const PluginSpec& p, const char* key) { return std::atof(p.get(key).c_str()); }

}  // namespace

struct gbmd_plugin {
  PluginSpec spec;
};

struct gbmd_sim {
  std::unique_ptr<Engine> eng;
};

struct gbmd_batch {
  std::unique_ptr<Engine> eng;
};

namespace gbmd {

std::string PluginSpec::get(const std::string& key) const {
  // ParamList::operator[] on a keyword that was never given yields an empty value
  // (liblpmd/core/paramlist.cc:38), which converts to 0.
  for (auto it = params.rbegin(); it != params.rend(); ++it)
    if (it->first == key) return it->second;
  return "";
}

PotParams finalize_potential(int kind, const double* v, int s1, int s2) {
  PotParams P;
  std::memset(&P, 0, sizeof(P));
  P.kind = kind;
  P.spc_sum = s1 + s2;
  P.int_n = P.int_m = -1;
  int np = (kind == POT_LJ) ? 3 : (kind == POT_FASTLJ) ? 4 : (kind == POT_SC || kind == POT_GUPTA) ? 6
         : (kind == POT_FS) ? 7 : 9;
  for (int k = 0; k < np; ++k) P.p[k] = v[k];
  if (kind == POT_FASTLJ) {
    P.cutoff = v[2];  // plugins/fastlj.cc:24; v[3] = bins (FP64 only: no mixed constants)
  } else if (kind == POT_LJ) {
    P.cutoff = v[2];
    const double s = v[0], e = v[1];
    P.f[0] = (float)(s * s);
    P.f[4] = (float)(s * s - (double)P.f[0]);  // low part of sigma^2 (double-float)
    P.f[1] = (float)(48.0 * e);
    P.f[2] = (float)(24.0 * e);
    P.f[3] = (float)(4.0 * e);
  } else if (kind == POT_SC) {
    const double e = v[0], a = v[1], n = v[2], m = v[3], c = v[4];
    P.cutoff = v[5];
    P.an = std::pow(a, n);  // plugins/suttonchen.cc:29-30
    P.am = std::pow(a, m);
    if (n == std::floor(n) && n >= 0 && n <= 64) P.int_n = (int)n;
    if (m == std::floor(m) && m >= 0 && m <= 64) P.int_m = (int)m;
    P.f[0] = (float)(e * P.an);
    P.f[1] = (float)(-n * e * P.an);
    P.f[2] = (float)(0.5 * m * c * e * P.am);
    P.f[3] = (float)P.am;
  } else if (kind == POT_GUPTA) {
    const double A = v[0], r0 = v[1], p = v[2], B = v[3], q = v[4];
    P.cutoff = v[5];  // plugins/gupta.cc:26
    P.f[0] = (float)A;
    P.f[1] = (float)(-p / r0);
    P.f[2] = (float)(-(A * p / r0));
    P.f[3] = (float)(B * q / r0);
    P.f[4] = (float)(-2.0 * q / r0);
    P.f[5] = (float)r0;
  } else {
    double c = (kind == POT_FS) ? v[5] : v[7];
    double d = (kind == POT_FS) ? v[6] : v[8];
    P.cutoff = (d >= c) ? d : c;  // plugins/finnissinclair.cc:27-30
    if (kind == POT_FS) {
      P.f[0] = (float)v[0];
      P.f[1] = (float)v[1];
      P.f[2] = (float)v[2];
      P.f[5] = (float)v[3];
      P.f[6] = (float)v[4];
    } else {
      for (int k = 0; k < 5; ++k) P.f[k] = (float)v[k];
      P.f[5] = (float)v[5];
      P.f[6] = (float)v[6];
    }
    P.f[7] = (float)c;
    P.f[8] = (float)d;
  }
  P.rc2 = P.cutoff * P.cutoff;
  P.f[12] = band_lo(P.rc2);
  P.f[13] = band_hi(P.rc2);
  return P;
}

PluginSpec make_plugin(const std::string& name, const std::string& args) {
  PluginSpec p;
  p.name = name;
  // Module::ProcessArguments (liblpmd/plugins/module.cc:77-103)
  std::istringstream in(args);
  std::string w;
  std::vector<std::string> words;
  while (in >> w) words.push_back(w);
  if (words.size() % 2) throw Error(GBMD_ERR_SYNTAX, "SyntaxError: Unexpected end of input while reading module arguments");
  for (size_t k = 0; k < words.size(); k += 2) p.params.emplace_back(words[k], words[k + 1]);
  auto has = [&](const char* k) { return !p.get(k).empty(); };
  auto defaulted = [&](const char* k, const char* def) {
    if (!has(k)) p.params.insert(p.params.begin(), {k, def});
  };
  if (name == "linkedcell") {
    p.kind = GBMD_KIND_CELLMANAGER;
    defaulted("cutoff", "7.0");
    defaulted("nx", "0");
    defaulted("ny", "0");
    defaulted("nz", "0");
    defaulted("mode", "noauto");
    defaulted("warn-outside", "true");
    p.cm.kind = CM_LINKEDCELL;
    p.cm.cutoff = num(p, "cutoff");
    p.cm.nx = std::atoi(p.get("nx").c_str());
    p.cm.ny = std::atoi(p.get("ny").c_str());
    p.cm.nz = std::atoi(p.get("nz").c_str());
    p.cm.mode_auto = (p.get("mode") == "auto" || p.get("mode") == "AUTO");  // linkedcell.cc:38-41
    if (has("skin")) p.cm.skin = num(p, "skin");
    p.cm.compat = (p.get("compat") == "true");
  } else if (name == "verletlist") {
    p.kind = GBMD_KIND_CELLMANAGER;
    bool each_given = has("each");
    defaulted("cutoff", "0.0");
    defaulted("extcutoff", "0.0");
    defaulted("maxneighbors", "80");
    defaulted("each", "5");
    p.cm.kind = CM_VERLETLIST;
    p.cm.cutoff = num(p, "cutoff");
    p.cm.maxneighbors = std::atol(p.get("maxneighbors").c_str());
    p.cm.each = std::atol(p.get("each").c_str());
    if (p.cm.each <= 0) throw Error(GBMD_ERR_PLUGIN, "verletlist: each must be positive");
    if (has("skin")) {
      p.cm.skin = num(p, "skin");
      p.cm.rebuild = each_given ? REBUILD_BOTH : REBUILD_SKIN;
    }
    if (has("rebuild")) {
      std::string r = p.get("rebuild");
      p.cm.rebuild = (r == "each") ? REBUILD_EACH : (r == "skin") ? REBUILD_SKIN : REBUILD_BOTH;
    }
  } else if (name == "lcbinary") {
    // plugins/lcbinary.cc:9-31: cutoff 7.0, nx ny nz 0, mode noauto; any zero count means auto
    p.kind = GBMD_KIND_CELLMANAGER;
    defaulted("cutoff", "7.0");
    defaulted("nx", "0");
    defaulted("ny", "0");
    defaulted("nz", "0");
    defaulted("mode", "noauto");
    p.cm.kind = CM_LCBINARY;
    p.cm.cutoff = num(p, "cutoff");
    p.cm.nx = std::atoi(p.get("nx").c_str());
    p.cm.ny = std::atoi(p.get("ny").c_str());
    p.cm.nz = std::atoi(p.get("nz").c_str());
    p.cm.mode_auto = p.cm.nx == 0 || p.cm.ny == 0 || p.cm.nz == 0 || p.get("mode") == "auto" || p.get("mode") == "AUTO";
    if (has("skin")) p.cm.skin = num(p, "skin");
  } else if (name == "minimumimage") {
    p.kind = GBMD_KIND_CELLMANAGER;
    defaulted("cutoff", "0.0");
    p.cm.kind = CM_MINIMUMIMAGE;
    p.cm.cutoff = num(p, "cutoff");
  } else if (name == "lennardjones" || name == "suttonchen" || name == "finnissinclair" ||
             name == "finnissinclair-ext" || name == "gupta" || name == "fastlj") {
    p.kind = GBMD_KIND_POTENTIAL;
    static const char* lj[] = {"sigma", "epsilon", "cutoff"};
    static const char* sc[] = {"e", "a", "n", "m", "c", "cutoff"};
    static const char* fs[] = {"c0", "c1", "c2", "A", "B", "c", "d"};
    static const char* fx[] = {"c0", "c1", "c2", "c3", "c4", "A", "B", "c", "d"};
    static const char* gu[] = {"A", "r0", "p", "B", "q", "cutoff"};  // plugins/gupta.cc:14-19
    static const char* fl[] = {"sigma", "epsilon", "cutoff", "bins"};  // plugins/fastlj.cc:15-19
    int kind = name == "lennardjones" ? POT_LJ : name == "suttonchen" ? POT_SC : name == "finnissinclair" ? POT_FS
             : name == "gupta" ? POT_GUPTA : name == "fastlj" ? POT_FASTLJ : POT_FSEXT;
    const char** keys = kind == POT_LJ ? lj : kind == POT_SC ? sc : kind == POT_FS ? fs : kind == POT_GUPTA ? gu
                      : kind == POT_FASTLJ ? fl : fx;
    int nk = kind == POT_LJ ? 3 : kind == POT_FASTLJ ? 4 : (kind == POT_SC || kind == POT_GUPTA) ? 6
           : kind == POT_FS ? 7 : 9;
    if (kind == POT_FASTLJ) defaulted("bins", "500");
    if (kind == POT_SC) defaulted("corrections", "false");
    double v[10] = {0};
    for (int k = 0; k < nk; ++k) v[k] = num(p, keys[k]);
    p.pot = finalize_potential(kind, v, -1, -1);
    if (has("precision")) {
      std::string pr = p.get("precision");
      if (pr == "mixed") p.precision = PREC_MIXED;
      else if (pr == "fp64") p.precision = PREC_FP64;
      else throw Error(GBMD_ERR_PLUGIN, name + ": precision must be mixed or fp64");
    }
  } else if (name == "velocityverlet" || name == "euler" || name == "leapfrog" || name == "verlet" ||
             name == "beeman" || name == "nosehoover") {
    // dt 1.0 and start 1 for all of them (plugins/velocityverlet.cc, euler.cc, leapfrog.cc,
    // verlet.cc, beeman.cc); nosehoover adds fmass (no default) and t 300.0 (nosehoover.cc:13-24)
    p.kind = GBMD_KIND_INTEGRATOR;
    defaulted("dt", "1.0");
    defaulted("start", "1");
    p.integ.kind = name == "velocityverlet" ? 0 : name == "euler" ? 1 : name == "leapfrog" ? 2
                 : name == "verlet" ? 3 : name == "beeman" ? 4 : 5;
    p.integ.dt = num(p, "dt");
    p.integ.start = std::atol(p.get("start").c_str());
    if (name == "nosehoover") {
      defaulted("t", "300.0");
      // an absent fmass reads as 0 in the reference and divides by zero: refused here
      if (!has("fmass")) throw Error(GBMD_ERR_PLUGIN, "PluginError: nosehoover: the fmass keyword is required");
      p.integ.fmass = num(p, "fmass");
      p.integ.t = num(p, "t");
      if (!(p.integ.fmass > 0.0)) throw Error(GBMD_ERR_PLUGIN, "PluginError: nosehoover: fmass must be positive");
    }
  } else {
    throw Error(GBMD_ERR_PLUGIN, "PluginError: no GPU implementation of plugin \"" + name + "\"");
  }
  if (!has("debug")) p.params.insert(p.params.begin(), {"debug", "stderr"});
  return p;
}

// Host FP64 functionals, evaluated exactly as the reference plugins write them.
void potential_eval(const PotParams& P, int what, const double* a, double* out) {
  const double* v = P.p;
  if (P.kind == POT_FASTLJ) {  // plugins/fastlj.cc:38-73: the table entry of the distance's bin
    const double sigma = v[0], epsilon = v[1], cutoff = v[2];
    const long bins = (long)v[3];
    double r = what == 0 ? a[0] : std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    long k = long(std::floor(bins * r / cutoff));
    if (what > 1) throw Error(GBMD_ERR_INVALID, "fastlj is a pair potential: only pairEnergy and pairForce");
    if (k < 0 || k >= bins) throw Error(GBMD_ERR_INVALID, "fastlj: distance outside the table");
    double rk = cutoff * double(k) / double(bins);
    double r6 = std::pow(sigma / rk, 6.0e0);
    double r12 = r6 * r6;
    if (what == 0) {
      out[0] = 4.0e0 * epsilon * (r12 - r6);
    } else {
      double ff = -48.0e0 * (epsilon / (rk * rk)) * (r12 - 0.50e0 * r6);
      for (int q = 0; q < 3; ++q) out[q] = a[q] * ff;
    }
    return;
  }
  if (P.kind == POT_LJ) {
    const double sigma = v[0], epsilon = v[1];
    if (what == 0) {  // plugins/lennardjones.cc:53-58
      double rtmp = sigma / a[0];
      double r6 = rtmp * rtmp * rtmp * rtmp * rtmp * rtmp;
      double r12 = r6 * r6;
      out[0] = 4.0e0 * epsilon * (r12 - r6);
    } else if (what == 1) {  // plugins/lennardjones.cc:60-67
      double rr2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
      double r6 = std::pow(sigma * sigma / rr2, 3.0e0);
      double r12 = r6 * r6;
      double ff = -48.0e0 * (epsilon / rr2) * (r12 - 0.50e0 * r6);
      for (int q = 0; q < 3; ++q) out[q] = a[q] * ff;
    } else {
      throw Error(GBMD_ERR_INVALID, "lennardjones is a pair potential: only pairEnergy and pairForce");
    }
    return;
  }
  auto rho_of = [&](double r) {
    if (P.kind == POT_GUPTA) return std::exp(-2.0e0 * v[4] * (r - v[1]) / v[1]);  // gupta.cc:56
    if (P.kind == POT_SC) return P.am * std::pow(1 / r, v[3]);
    if (P.kind == POT_FS) {
      const double B = v[4], d = v[6];
      return r <= d ? ((r - d) * (r - d)) * (1.0e0 + B * (r - d) / d) : 0.0;
    }
    const double B = v[6], d = v[8];
    double rd = r - d;
    return r <= d ? (rd * rd) * (1.0e0 + B * B * rd * rd) : 0.0;
  };
  if (what == 0) {
    double r = a[0];
    if (P.kind == POT_GUPTA) {
      out[0] = v[0] * std::exp(-v[2] * (r - v[1]) / v[1]);  // gupta.cc:54
    } else if (P.kind == POT_SC) {
      out[0] = v[0] * P.an * std::pow(1 / r, v[2]);
    } else if (P.kind == POT_FS) {
      const double c0 = v[0], c1 = v[1], c2 = v[2], c = v[5];
      out[0] = r <= c ? (r - c) * (r - c) * (c0 + c1 * r + c2 * r * r) : 0.0;
    } else {
      const double c = v[7];
      double r2 = r * r;
      out[0] = r <= c ? (r - c) * (r - c) * (v[0] + v[1] * r + v[2] * r2 + v[3] * r2 * r + v[4] * r2 * r2) : 0.0;
    }
  } else if (what == 2) {
    out[0] = rho_of(a[0]);
  } else if (what == 3) {
    double A = P.kind == POT_SC ? v[4] * v[0] : (P.kind == POT_FS || P.kind == POT_GUPTA) ? v[3] : v[5];
    out[0] = P.kind == POT_SC ? -v[4] * v[0] * std::sqrt(a[0]) : -A * std::sqrt(a[0]);
  } else if (what == 1 || what == 4 || what == 5 || what == 6) {
    // 1, 4: from r_ij; 5, 6: from the unit vector and the modulus as the reference's
    // PairForce(normrij, rmod) / ManyBodies(normrij, rhoi, rhoj, rmod) receive them
    const bool given = what >= 5;
    double r = given ? a[what == 5 ? 3 : 5] : std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double nrm[3] = {given ? a[0] : a[0] / r, given ? a[1] : a[1] / r, given ? a[2] : a[2] / r};
    double s = 0.0;
    if (what == 1 || what == 5) {
      if (P.kind == POT_GUPTA) {  // gupta.cc:60-62
        s = -(v[0] * v[2] / v[1]) * std::exp(-v[2] * (r - v[1]) / v[1]);
      } else if (P.kind == POT_SC) {
        double ir = 1.0e0 / r;
        s = -v[2] * v[0] * P.an * std::pow(ir, v[2] + 1);
      } else if (P.kind == POT_FS) {
        const double c0 = v[0], c1 = v[1], c2 = v[2], c = v[5];
        if (r <= c) s = 2.0e0 * (r - c) * (c0 + c1 * r + c2 * r * r) + (r - c) * (r - c) * (c1 + 2.0e0 * c2 * r);
      } else {
        const double c = v[7];
        if (r <= c) {
          double r2 = r * r, rc = r - c;
          s = 2.0e0 * rc * (v[0] + v[1] * r + v[2] * r2 + v[3] * r2 * r + v[4] * r2 * r2) +
              (v[1] + 2.0e0 * v[2] * r + 3.0e0 * v[3] * r2 + 4.0e0 * v[4] * r2 * r) * rc * rc;
        }
      }
    } else {
      const double rhoi = a[3], rhoj = a[4];
      if (P.kind == POT_GUPTA) {  // gupta.cc:64-70
        s = (v[3] * v[4] / v[1]) * ((1.0e0 / std::sqrt(rhoi)) + (1.0e0 / std::sqrt(rhoj))) *
            std::exp(-2.0e0 * v[4] * (r - v[1]) / v[1]);
      } else if (P.kind == POT_SC) {
        double ir = 1.0e0 / r;
        s = 0.5 * v[3] * v[4] * v[0] * ((1 / std::sqrt(rhoi)) + 1 / (std::sqrt(rhoj))) * P.am * std::pow(ir, v[3] + 1);
      } else if (P.kind == POT_FS) {
        const double A = v[3], B = v[4], d = v[6];
        if (r <= d) {
          double t1 = ((1.0e0 / std::sqrt(rhoi)) + (1.0e0 / std::sqrt(rhoj))) * A / 2.0e0;
          double t2 = 2.0e0 * (r - d) + 3.0e0 * B * (r - d) * (r - d) / d;
          s = -t1 * t2;
        }
      } else {
        const double A = v[5], B = v[6], d = v[8];
        if (r <= d) {
          double rd = r - d;
          double t1 = A * 0.5e0 * ((1.0e0 / std::sqrt(rhoi)) + (1.0e0 / std::sqrt(rhoj)));
          double t2 = 2.0e0 * rd + 4.0e0 * B * B * rd * rd * rd;
          s = -t1 * t2;
        }
      }
    }
    for (int q = 0; q < 3; ++q) out[q] = s * nrm[q];
  } else {
    throw Error(GBMD_ERR_INVALID, "unknown functional index");
  }
}

}  // namespace gbmd

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------

extern "C" {

const char* gbmd_last_error(void) { return g_last_error.c_str(); }

int gbmd_abi_version(void) { return 1; }

gbmd_status gbmd_device_count(int* count) {
  if (!count) return fail(GBMD_ERR_INVALID, "null argument");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return GBMD_OK;
}

gbmd_status gbmd_plugin_create(const char* name, const char* args, gbmd_plugin** out) {
  if (!name || !out) return fail(GBMD_ERR_INVALID, "null argument");
  return guarded([&] {
    auto* p = new gbmd_plugin;
    try {
      p->spec = make_plugin(name, args ? args : "");
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

void gbmd_plugin_destroy(gbmd_plugin* plugin) { delete plugin; }

gbmd_status gbmd_plugin_kind(const gbmd_plugin* p, int* kind) {
  if (!p || !kind) return fail(GBMD_ERR_INVALID, "null argument");
  *kind = p->spec.kind;
  return GBMD_OK;
}

gbmd_status gbmd_plugin_param(const gbmd_plugin* p, const char* key, char* buf, size_t len) {
  if (!p || !key || !buf) return fail(GBMD_ERR_INVALID, "null argument");
  std::string v = p->spec.get(key);
  if (v.size() + 1 > len) return fail(GBMD_ERR_CAPACITY, "buffer too small");
  std::memcpy(buf, v.c_str(), v.size() + 1);
  return GBMD_OK;
}

gbmd_status gbmd_plugin_cutoff(const gbmd_plugin* p, double* cutoff) {
  if (!p || !cutoff) return fail(GBMD_ERR_INVALID, "null argument");
  if (p->spec.kind == GBMD_KIND_POTENTIAL)
    *cutoff = p->spec.pot.cutoff;
  else if (p->spec.kind == GBMD_KIND_CELLMANAGER)
    *cutoff = p->spec.cm.cutoff;
  else
    return fail(GBMD_ERR_INVALID, "an integrator has no cutoff");
  return GBMD_OK;
}

gbmd_status gbmd_potential_eval(const gbmd_plugin* p, int what, const double* args, double* out) {
  if (!p || !args || !out) return fail(GBMD_ERR_INVALID, "null argument");
  if (p->spec.kind != GBMD_KIND_POTENTIAL) return fail(GBMD_ERR_INVALID, "not a potential");
  return guarded([&] { potential_eval(p->spec.pot, what, args, out); });
}

gbmd_status gbmd_selftest_bounded_wait(int device, int64_t polls, int* gave_up) {
  if (!gave_up) return fail(GBMD_ERR_INVALID, "null argument");
  return guarded([&] { *gave_up = wait_selftest(device, (long long)polls); });
}

gbmd_status gbmd_pair_forces_static(const gbmd_plugin* p, const double* pos, int n, const double* box, double* force,
                                    double* out, void* stream) {
  if (!p || !pos || !box || !force || !out) return fail(GBMD_ERR_INVALID, "null argument");
  if (p->spec.kind != GBMD_KIND_POTENTIAL) return fail(GBMD_ERR_INVALID, "not a potential");
  return guarded([&] {
    PotParams P = p->spec.pot;
    P.spc_sum = -2;  // every pair interacts
    pair_forces_static(P, pos, n, box, force, out, stream);
  });
}

// ---- simulation ----

gbmd_status gbmd_sim_create(int device, int64_t natoms, const double cell[3], gbmd_sim** out) {
  if (!cell || !out) return fail(GBMD_ERR_INVALID, "null argument");
  return guarded([&] {
    auto* s = new gbmd_sim;
    try {
      s->eng.reset(new Engine(device, {natoms}, {{cell[0], cell[1], cell[2]}}));
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

void gbmd_sim_destroy(gbmd_sim* sim) { delete sim; }

#define SIM_GUARD(body)                                                 \
  if (!sim) return fail(GBMD_ERR_INVALID, "null simulation");           \
  return guarded([&] { body; })

gbmd_status gbmd_sim_set_atoms(gbmd_sim* sim, const double* pos, const double* vel, const double* acc,
                               const int32_t* Z, const double* mass) {
  SIM_GUARD(sim->eng->set_atoms(0, pos, vel, acc, Z, mass));
}

gbmd_status gbmd_sim_set_flags(gbmd_sim* sim, const uint8_t* flags) { SIM_GUARD(sim->eng->set_flags(0, flags)); }

gbmd_status gbmd_sim_get_atoms(gbmd_sim* sim, double* pos, double* vel, double* acc) {
  SIM_GUARD(sim->eng->get_atoms(0, pos, vel, acc));
}

static void need_kind(const gbmd_plugin* p, int kind, const char* what) {
  if (!p) throw Error(GBMD_ERR_INVALID, "null plugin");
  if (p->spec.kind != kind) throw Error(GBMD_ERR_INVALID, std::string("plugin \"") + p->spec.name + "\" is not a " + what);
}

static void apply_cm(Engine& e, const gbmd_plugin* p) {
  need_kind(p, GBMD_KIND_CELLMANAGER, "cell manager");
  e.set_cell_manager(p->spec.cm);
  if (p->spec.cm.kind == CM_VERLETLIST) e.set_option("maxneighbors_cap", std::to_string(p->spec.cm.maxneighbors));
}

static void apply_pot(Engine& e, const gbmd_plugin* p, int s1, int s2) {
  need_kind(p, GBMD_KIND_POTENTIAL, "potential");
  PotParams P = p->spec.pot;
  P.spc_sum = s1 + s2;
  e.add_potential(P);
  if (p->spec.precision >= 0) e.set_precision(p->spec.precision);
}

static void apply_integ(Engine& e, const gbmd_plugin* p) {
  need_kind(p, GBMD_KIND_INTEGRATOR, "integrator");
  e.set_integrator(p->spec.integ);
}

gbmd_status gbmd_sim_set_cell_manager(gbmd_sim* sim, const gbmd_plugin* cm) { SIM_GUARD(apply_cm(*sim->eng, cm)); }

gbmd_status gbmd_sim_add_potential(gbmd_sim* sim, const gbmd_plugin* pot, int s1, int s2) {
  SIM_GUARD(apply_pot(*sim->eng, pot, s1, s2));
}

gbmd_status gbmd_sim_set_integrator(gbmd_sim* sim, const gbmd_plugin* integ) {
  SIM_GUARD(apply_integ(*sim->eng, integ));
}

gbmd_status gbmd_sim_set_precision(gbmd_sim* sim, int precision) { SIM_GUARD(sim->eng->set_precision(precision)); }

gbmd_status gbmd_sim_set_option(gbmd_sim* sim, const char* key, const char* value) {
  if (!key || !value) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(sim->eng->set_option(key, value));
}

gbmd_status gbmd_sim_update_forces(gbmd_sim* sim) { SIM_GUARD(sim->eng->update_forces()); }

gbmd_status gbmd_sim_do_steps(gbmd_sim* sim, int64_t nsteps) {
  if (nsteps < 0) return fail(GBMD_ERR_INVALID, "negative step count");
  SIM_GUARD(sim->eng->do_steps(nsteps));
}

gbmd_status gbmd_sim_synchronize(gbmd_sim* sim) { SIM_GUARD(sim->eng->synchronize()); }

gbmd_status gbmd_sim_thermo(gbmd_sim* sim, gbmd_thermo* out) {
  if (!out) return fail(GBMD_ERR_INVALID, "null argument");
  static_assert(sizeof(gbmd_thermo) == 22 * sizeof(double), "thermo layout");
  SIM_GUARD(sim->eng->thermo(0, (double*)out));
}

gbmd_status gbmd_sim_thermo_log(gbmd_sim* sim, gbmd_thermo* out, int64_t cap, int64_t* count) {
  if (!out || !count) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(*count = sim->eng->thermo_log(0, (double*)out, cap));
}

static void copy_stats(const Stats& s, gbmd_stats* out) {
  out->steps = s.steps;
  out->force_evaluations = s.force_evaluations;
  out->list_rebuilds = s.list_rebuilds;
  out->kernel_launches = s.kernel_launches;
  out->max_neighbors = s.max_neighbors;
  out->list_capacity = s.list_capacity;
  out->neighbor_mode = s.neighbor_mode;
  for (int q = 0; q < 3; ++q) out->cell_grid[q] = s.cell_grid[q];
  out->list_radius = s.list_radius;
  out->device_bytes = s.device_bytes;
  out->fp_guard_rechecks = s.fp_guard_rechecks;
  out->force_ms = s.force_ms;
  out->force_launches = s.force_launches;
  out->drift_ms = s.drift_ms;
  out->drift_launches = s.drift_launches;
  out->rebuild_ms = s.rebuild_ms;
  out->rebuild_launches = s.rebuild_launches;
}

gbmd_status gbmd_sim_stats(gbmd_sim* sim, gbmd_stats* out) {
  if (!out) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(copy_stats(sim->eng->stats(), out));
}

gbmd_status gbmd_sim_stream(gbmd_sim* sim, void** stream) {
  if (!stream) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(*stream = sim->eng->stream());
}

gbmd_status gbmd_sim_neighbors(gbmd_sim* sim, int full, double rcut, int64_t* counts, int64_t* idx, int64_t cap,
                               int64_t* total) {
  SIM_GUARD(sim->eng->neighbors(0, full, rcut, counts, idx, cap, total));
}

gbmd_status gbmd_sim_cell_sort(gbmd_sim* sim, const int32_t n[3], int64_t* cell, int64_t* order) {
  if (!n) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(sim->eng->cell_sort(0, n, cell, order));
}

// ---- batch ----

gbmd_status gbmd_batch_create(int device, int nsys, const int64_t* natoms, const double* cells, gbmd_batch** out) {
  if (!natoms || !cells || !out || nsys <= 0) return fail(GBMD_ERR_INVALID, "bad argument");
  return guarded([&] {
    std::vector<int64_t> na(natoms, natoms + nsys);
    std::vector<std::array<double, 3>> cl(nsys);
    for (int s = 0; s < nsys; ++s) cl[s] = {cells[3 * s], cells[3 * s + 1], cells[3 * s + 2]};
    auto* b = new gbmd_batch;
    try {
      b->eng.reset(new Engine(device, na, cl));
    } catch (...) {
      delete b;
      throw;
    }
    *out = b;
  });
}

void gbmd_batch_destroy(gbmd_batch* batch) { delete batch; }

#define BATCH_GUARD(body)                                           \
  if (!batch) return fail(GBMD_ERR_INVALID, "null batch");          \
  return guarded([&] { body; })

gbmd_status gbmd_batch_set_atoms(gbmd_batch* batch, int sys, const double* pos, const double* vel, const int32_t* Z,
                                 const double* mass) {
  BATCH_GUARD(batch->eng->set_atoms(sys, pos, vel, nullptr, Z, mass));
}

gbmd_status gbmd_sim_checkpoint_size(gbmd_sim* sim, size_t* bytes) {
  if (!bytes) return fail(GBMD_ERR_INVALID, "null argument");
  SIM_GUARD(*bytes = sim->eng->checkpoint_size());
}
gbmd_status gbmd_sim_checkpoint_save(gbmd_sim* sim, void* buf, size_t bytes) {
  SIM_GUARD(sim->eng->checkpoint_save(buf, bytes));
}
gbmd_status gbmd_sim_checkpoint_load(gbmd_sim* sim, const void* buf, size_t bytes) {
  SIM_GUARD(sim->eng->checkpoint_load(buf, bytes));
}
gbmd_status gbmd_batch_checkpoint_size(gbmd_batch* batch, size_t* bytes) {
  if (!bytes) return fail(GBMD_ERR_INVALID, "null argument");
  BATCH_GUARD(*bytes = batch->eng->checkpoint_size());
}
gbmd_status gbmd_batch_checkpoint_save(gbmd_batch* batch, void* buf, size_t bytes) {
  BATCH_GUARD(batch->eng->checkpoint_save(buf, bytes));
}
gbmd_status gbmd_batch_checkpoint_load(gbmd_batch* batch, const void* buf, size_t bytes) {
  BATCH_GUARD(batch->eng->checkpoint_load(buf, bytes));
}

gbmd_status gbmd_sim_scale_velocities(gbmd_sim* sim, int mode, double target, double dt_over_tau) {
  SIM_GUARD(sim->eng->scale_velocities(-1, mode, target, dt_over_tau));
}
gbmd_status gbmd_batch_scale_velocities(gbmd_batch* batch, int sys, int mode, double target, double dt_over_tau) {
  BATCH_GUARD(batch->eng->scale_velocities(sys, mode, target, dt_over_tau));
}

gbmd_status gbmd_batch_set_active(gbmd_batch* batch, int sys, int active) {
  BATCH_GUARD(batch->eng->set_active(sys, active != 0));
}

gbmd_status gbmd_batch_get_atoms(gbmd_batch* batch, int sys, double* pos, double* vel, double* acc) {
  BATCH_GUARD(batch->eng->get_atoms(sys, pos, vel, acc));
}

gbmd_status gbmd_batch_set_cell_manager(gbmd_batch* batch, const gbmd_plugin* cm) { BATCH_GUARD(apply_cm(*batch->eng, cm)); }

gbmd_status gbmd_batch_add_potential(gbmd_batch* batch, const gbmd_plugin* pot, int s1, int s2) {
  BATCH_GUARD(apply_pot(*batch->eng, pot, s1, s2));
}

gbmd_status gbmd_batch_set_integrator(gbmd_batch* batch, const gbmd_plugin* integ) {
  BATCH_GUARD(apply_integ(*batch->eng, integ));
}

gbmd_status gbmd_batch_set_precision(gbmd_batch* batch, int precision) { BATCH_GUARD(batch->eng->set_precision(precision)); }

gbmd_status gbmd_batch_set_option(gbmd_batch* batch, const char* key, const char* value) {
  if (!key || !value) return fail(GBMD_ERR_INVALID, "null argument");
  BATCH_GUARD(batch->eng->set_option(key, value));
}

gbmd_status gbmd_batch_update_forces(gbmd_batch* batch) { BATCH_GUARD(batch->eng->update_forces()); }

gbmd_status gbmd_batch_do_steps(gbmd_batch* batch, int64_t nsteps) {
  if (nsteps < 0) return fail(GBMD_ERR_INVALID, "negative step count");
  BATCH_GUARD(batch->eng->do_steps(nsteps));
}

gbmd_status gbmd_batch_synchronize(gbmd_batch* batch) { BATCH_GUARD(batch->eng->synchronize()); }

gbmd_status gbmd_batch_thermo(gbmd_batch* batch, int sys, gbmd_thermo* out) {
  if (!out) return fail(GBMD_ERR_INVALID, "null argument");
  BATCH_GUARD(batch->eng->thermo(sys, (double*)out));
}

gbmd_status gbmd_batch_stats(gbmd_batch* batch, gbmd_stats* out) {
  if (!out) return fail(GBMD_ERR_INVALID, "null argument");
  BATCH_GUARD(copy_stats(batch->eng->stats(), out));
}

gbmd_status gbmd_batch_stream(gbmd_batch* batch, void** stream) {
  if (!stream) return fail(GBMD_ERR_INVALID, "null argument");
  BATCH_GUARD(*stream = batch->eng->stream());
}

gbmd_status gbmd_batch_neighbors(gbmd_batch* batch, int sys, int full, double rcut, int64_t* counts, int64_t* idx,
                                 int64_t cap, int64_t* total) {
  BATCH_GUARD(batch->eng->neighbors(sys, full, rcut, counts, idx, cap, total));
}

}  // extern "C"

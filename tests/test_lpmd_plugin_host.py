"""The LPMD-side binding, host side: the plugins of lpmd2_gb300/lpmd_plugin/ compiled against
the reference's liblpmd headers and loaded through liblpmd's own PluginLoader (the reference's
sources, built by oracle/Makefile's `ref` target), in a process that has no GPU.

The `gbmd` integrator plugin (gbmd.cc): an lpmd::Integrator reachable by dynamic_cast, its
keywords and defaults processed by Module::ProcessArguments, a keyword without a value raising
the reference's SyntaxError.

The GPU plugins under LPMD's own names (plugins.cc, one .so per name): loaded beside the
reference plugin of the same name, each is the same kind of object with the same keywords and
defaults; the host functionals (pairEnergy, pairForce, rhoij, F, PairForce, ManyBodies) equal
the reference's bit for bit; and a simulation wired through liblpmd (SetCellManager,
UpdateForces, DoStep, BuildNeighborList) reaches libgbmd, whose "no CUDA device" status comes
back as lpmd::RuntimeError.  Skipped where the reference checkout or its build is absent.
"""
import os
import subprocess
from pathlib import Path

import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
REF = oracle.reference_source()  # $LPMD_REFERENCE or the checkout the reference build used
REF_LIB = ROOT / "oracle" / "_ref" / "libref_driver.so"
GBMD_LIB = ROOT / "lpmd2_gb300" / "libgbmd.so"

HARNESS = r'''
#include <lpmd/error.h>
#include <lpmd/integrator.h>
#include <lpmd/plugin.h>
#include <cstdio>
#include <string>

int main(int argc, char** argv) {
  lpmd::Plugin* p = lpmd::PluginLoader(argv[1], "dt 2.5 precision fp64");
  lpmd::Integrator* integ = dynamic_cast<lpmd::Integrator*>(p);
  lpmd::Plugin& q = *p;
  std::printf("name=%s dt=%s precision=%s device=%s sync=%s scheme=%s integrator=%d\n", q.Name().c_str(),
              std::string(q["dt"]).c_str(), std::string(q["precision"]).c_str(),
              std::string(q["device"]).c_str(), std::string(q["sync-each"]).c_str(),
              std::string(q["scheme"]).c_str(), integ != nullptr);
  lpmd::Plugin& nh = *lpmd::PluginLoader(argv[1], "scheme nosehoover fmass 1e9 t 120");
  std::printf("scheme=%s fmass=%s t=%s\n", std::string(nh["scheme"]).c_str(), std::string(nh["fmass"]).c_str(),
              std::string(nh["t"]).c_str());
  try {
    lpmd::PluginLoader(argv[1], "dt 1.0 device");
    std::printf("no error\n");
  } catch (lpmd::Error& e) {
    std::printf("error: %s\n", e.what());
  }
  return 0;
}
'''


@pytest.fixture(scope="module")
def plugin(tmp_path_factory):
    if REF is None or not (REF / "liblpmd" / "lpmd" / "plugin.h").exists():
        pytest.skip("no lpmd2 reference checkout named (set LPMD_REFERENCE)")
    if not REF_LIB.exists() or not GBMD_LIB.exists():
        pytest.skip("reference build or libgbmd.so not built (run __graft_entry__.build())")
    subprocess.run(["make", "-s", "-C", str(ROOT / "lpmd2_gb300" / "lpmd_plugin"), f"LPMD={REF}"], check=True)
    so = ROOT / "lpmd2_gb300" / "_build" / "lpmd_plugin" / "gbmd.so"
    d = tmp_path_factory.mktemp("harness")
    (d / "h.cpp").write_text(HARNESS)
    exe = d / "h"
    subprocess.run(["g++", "-std=c++17", "-O1", str(d / "h.cpp"), "-I", str(ROOT / "oracle" / "_ref"), "-I",
                    str(REF / "liblpmd"), "-L", str(REF_LIB.parent), "-lref_driver", "-ldl",
                    f"-Wl,-rpath,{REF_LIB.parent}", "-o", str(exe)], check=True)
    return so, exe


def test_plugin_loads_through_lpmd(plugin):
    so, exe = plugin
    env = dict(os.environ, LD_LIBRARY_PATH=f"{GBMD_LIB.parent}:{os.environ.get('LD_LIBRARY_PATH', '')}")
    out = subprocess.run([str(exe), str(so)], capture_output=True, text=True, env=env, timeout=60)
    assert out.returncode == 0, out.stderr
    first, nh, second = out.stdout.splitlines()[:3]
    assert first == "name=gbmd dt=2.5 precision=fp64 device=0 sync=1 scheme=velocityverlet integrator=1"
    assert nh == "scheme=nosehoover fmass=1e9 t=120"
    assert second.startswith("error:")


# --------------------------------------------------------------------------------------------
# The GPU plugins under LPMD's own names (lpmd2_gb300/lpmd_plugin/plugins.cc)
# --------------------------------------------------------------------------------------------

NAMED = ["lennardjones", "fastlj", "suttonchen", "finnissinclair", "finnissinclair-ext", "gupta", "linkedcell",
         "verletlist", "minimumimage", "lcbinary", "velocityverlet"]

NAMED_HARNESS = r'''
#include <lpmd/atom.h>
#include <lpmd/cellmanager.h>
#include <lpmd/combinedpotential.h>
#include <lpmd/error.h>
#include <lpmd/integrator.h>
#include <lpmd/metalpotential.h>
#include <lpmd/pairpotential.h>
#include <lpmd/plugin.h>
#include <lpmd/simulationbuilder.h>
#include <lpmd/util.h>
#include <runtime/runtime_context.h>
#include <cstdio>
#include <string>

using namespace lpmd;

// the reference plugins, compiled into libref_driver.so with their entry points renamed
#define REF(n) extern "C" Plugin* create_##n(std::string);
REF(lennardjones) REF(fastlj) REF(suttonchen) REF(finnissinclair) REF(finnissinclair_ext) REF(gupta)
REF(linkedcell) REF(verletlist) REF(minimumimage) REF(lcbinary) REF(velocityverlet)

struct Case { const char* name; const char* args; Plugin* (*ref)(std::string); };
const Case cases[] = {
  {"lennardjones", "sigma 3.405 epsilon 0.0103 cutoff 8.5", create_lennardjones},
  {"fastlj", "sigma 3.405 epsilon 0.0103 cutoff 8.5", create_fastlj},
  {"suttonchen", "e 0.012382 a 3.61 n 9 m 6 c 39.432 cutoff 7.22", create_suttonchen},
  {"finnissinclair", "c0 1.2371147 c1 -0.3592185 c2 -0.0385607 A 1.828905 B 1.8 c 3.40 d 3.569745", create_finnissinclair},
  {"finnissinclair-ext", "c0 47.13 c1 -33.77 c2 6.25 c3 -0.0122 c4 0.0001 A 1.848 B 0.5 c 3.25 d 4.1", create_finnissinclair_ext},
  {"gupta", "A 0.2061 r0 2.884 p 10.229 B 1.790 q 4.036 cutoff 6.0", create_gupta},
  {"linkedcell", "cutoff 8.5 nx 6 ny 6 nz 6", create_linkedcell},
  {"verletlist", "cutoff 8.5 maxneighbors 128", create_verletlist},
  {"minimumimage", "cutoff 8.5", create_minimumimage},
  {"lcbinary", "cutoff 8.5", create_lcbinary},
  {"velocityverlet", "dt 2.0", create_velocityverlet},
};

std::string kinds(Plugin* p) {
  std::string k;
  if (dynamic_cast<PairPotential*>(p)) k += "pair ";
  if (dynamic_cast<MetalPotential*>(p)) k += "metal ";
  if (dynamic_cast<CellManager*>(p)) k += "cellmanager ";
  if (dynamic_cast<Integrator*>(p)) k += "integrator ";
  return k;
}

std::string keywords(Plugin* p) {  // the reference's keywords with their values, in its order
  std::string out;
  Array<std::string> kw = StringSplit(p->Keywords());
  for (long k = 0; k < kw.Size(); ++k) {
    if (kw[k] == "precision" || kw[k] == "sync-each" || kw[k] == "debug") continue;
    out += kw[k] + "=" + std::string((*p)[kw[k]]) + " ";
  }
  return out;
}

int main(int argc, char** argv) {
  const std::string dir = argv[1];
  for (const Case& c : cases) {
    Plugin* g = PluginLoader(dir + "/" + c.name + ".so", c.args);
    Plugin* r = c.ref(c.args);
    std::printf("plugin %s | %s| %s| %s| %s| %s\n", c.name, g->Name().c_str(), kinds(g).c_str(), kinds(r).c_str(),
                keywords(g).c_str(), keywords(r).c_str());
    if (PairPotential* gp = dynamic_cast<PairPotential*>(g)) {
      PairPotential* rp = dynamic_cast<PairPotential*>(r);
      for (double x : {3.1, 3.82, 4.4, 6.5, 8.2}) {
        Vector v(x * 0.48, -x * 0.6, x * 0.64);
        Vector fg = gp->pairForce(v), fr = rp->pairForce(v);
        std::printf("pair %s %a %a %a %a %a %a %a %a\n", c.name, gp->pairEnergy(x), rp->pairEnergy(x),
                    fg[0], fr[0], fg[1], fr[1], fg[2], fr[2]);
      }
      std::printf("cutoff %s %a %a\n", c.name, gp->GetCutoff(), rp->GetCutoff());
    }
    if (MetalPotential* gm = dynamic_cast<MetalPotential*>(g)) {
      MetalPotential* rm = dynamic_cast<MetalPotential*>(r);
      for (double x : {2.2, 2.55, 3.0, 3.5}) {
        Vector n(0.48, -0.6, 0.64);
        Vector pg = gm->PairForce(n, x), pr = rm->PairForce(n, x);
        Vector mg = gm->ManyBodies(n, 31.5, 29.25, x), mr = rm->ManyBodies(n, 31.5, 29.25, x);
        std::printf("metal %s %a %a %a %a %a %a %a %a %a %a %a %a\n", c.name, gm->pairEnergy(x), rm->pairEnergy(x),
                    gm->rhoij(x), rm->rhoij(x), gm->F(31.5), rm->F(31.5), pg[0], pr[0], pg[2], pr[2], mg[1], mr[1]);
      }
      std::printf("cutoff %s %a %a\n", c.name, gm->GetCutoff(), rm->GetCutoff());
    }
  }
  // a Simulation wired like a control file would wire it, driven up to the device call
  static RuntimeContext context;
  Simulation& md = SimulationBuilder::CreateFixedOrthogonal(context, 32, Atom("Ar"));
  md.Cell()[0] = 21.04 * e1;
  md.Cell()[1] = 21.04 * e2;
  md.Cell()[2] = 21.04 * e3;
  for (long i = 0; i < 32; ++i)
    md.Atoms()[i].Position() = Vector(0.6 * (i % 4) * 5.26, 0.6 * ((i / 4) % 4) * 5.26, 0.6 * (i / 16) * 5.26);
  CellManager& cm = *dynamic_cast<CellManager*>(PluginLoader(dir + "/linkedcell.so", "cutoff 8.5 nx 2 ny 2 nz 2"));
  md.SetCellManager(cm);  // calls UpdateCell: no device work
  std::printf("setcellmanager ok\n");
  Potential& lj = *dynamic_cast<Potential*>(PluginLoader(dir + "/lennardjones.so", "sigma 3.405 epsilon 0.0103 cutoff 8.5"));
  lj.SetValidSpecies(-1, -1);
  md.Potentials().Append(lj);
  Integrator& vv = *dynamic_cast<Integrator*>(PluginLoader(dir + "/velocityverlet.so", "dt 2.0"));
  md.SetIntegrator(vv);
  try {
    md.Potentials().Initialize(md);
    md.Potentials().UpdateForces(md);
    std::printf("updateforces no error\n");
  } catch (RuntimeError& e) {
    std::printf("updateforces RuntimeError: %s\n", e.what());
  } catch (Error& e) {
    std::printf("updateforces other error: %s\n", e.what());
  }
  try {
    md.DoStep();
    std::printf("dostep no error\n");
  } catch (RuntimeError& e) {
    std::printf("dostep RuntimeError: %s\n", e.what());
  } catch (Error& e) {
    std::printf("dostep other error: %s\n", e.what());
  }
  try {
    NeighborList nl;
    cm.BuildNeighborList(md, 0, nl, true, 8.5);
    std::printf("neighbors no error\n");
  } catch (RuntimeError& e) {
    std::printf("neighbors RuntimeError: %s\n", e.what());
  } catch (Error& e) {
    std::printf("neighbors other error: %s\n", e.what());
  }
  // a keyword without a value: Module::ProcessArguments throws SyntaxError, as with the
  // reference plugin (liblpmd/plugins/module.cc:99-103)
  for (const char* lib : {"/suttonchen.so", "SC"}) {
    try {
      if (lib[0] == '/')
        PluginLoader(dir + lib, "e 0.01 a 3.61 n 9 m 6 c 39 cutoff");
      else
        create_suttonchen("e 0.01 a 3.61 n 9 m 6 c 39 cutoff");
      std::printf("bad-args %s no error\n", lib);
    } catch (SyntaxError& e) {
      std::printf("bad-args %s SyntaxError\n", lib[0] == '/' ? "gpu" : "ref");
    }
  }
  return 0;
}
'''


@pytest.fixture(scope="module")
def named_plugins(tmp_path_factory):
    if REF is None or not (REF / "liblpmd" / "lpmd" / "plugin.h").exists():
        pytest.skip("no lpmd2 reference checkout named (set LPMD_REFERENCE)")
    if not REF_LIB.exists() or not GBMD_LIB.exists():
        pytest.skip("reference build or libgbmd.so not built (run __graft_entry__.build())")
    subprocess.run(["make", "-s", "-C", str(ROOT / "lpmd2_gb300" / "lpmd_plugin"), f"LPMD={REF}"], check=True)
    plugdir = ROOT / "lpmd2_gb300" / "_build" / "lpmd_plugin" / "plugins"
    d = tmp_path_factory.mktemp("named")
    (d / "h.cpp").write_text(NAMED_HARNESS)
    exe = d / "h"
    subprocess.run(["g++", "-std=c++17", "-O1", str(d / "h.cpp"), "-I", str(ROOT / "oracle" / "_ref"), "-I",
                    str(REF / "liblpmd"), "-L", str(REF_LIB.parent), "-lref_driver", "-ldl",
                    f"-Wl,-rpath,{REF_LIB.parent}", "-o", str(exe)], check=True)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")  # the host path up to the device call
    out = subprocess.run([str(exe), str(plugdir)], capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout.splitlines()


def test_named_plugins_match_the_reference_interfaces(named_plugins):
    """Every GPU plugin loads through liblpmd's PluginLoader under the reference's name, is the
    same kind of object (dynamic_cast to PairPotential / MetalPotential / CellManager /
    Integrator) and has the reference plugin's keywords with the same values and defaults."""
    rows = {ln.split()[1]: ln for ln in named_plugins if ln.startswith("plugin ")}
    assert sorted(rows) == sorted(NAMED)
    for name, ln in rows.items():
        _, gname, gkind, rkind, gkw, rkw = [x.strip() for x in ln.split(" ", 1)[1].split("|")]
        assert gname == name
        assert gkind == rkind and gkind, ln
        assert gkw == rkw, ln


def test_named_potentials_host_functionals_are_the_references_bit_for_bit(named_plugins):
    """pairEnergy / pairForce (pair) and pairEnergy / rhoij / F / PairForce / ManyBodies (metal),
    which host properties call, equal the reference plugin's in every bit (printed as %a)."""
    n = 0
    for ln in named_plugins:
        if ln.startswith(("pair ", "metal ", "cutoff ")):
            v = ln.split()[2:]
            assert v[0::2] == v[1::2], ln
            n += 1
    assert n >= 2 * 5 + 4 * 4 + 6


def test_named_plugins_drive_a_simulation_up_to_the_device(named_plugins):
    """SetCellManager / Potentials().UpdateForces / DoStep / BuildNeighborList through liblpmd on
    a host without a GPU: SetCellManager does no device work; the others reach libgbmd and its
    "no CUDA device" status comes back as lpmd::RuntimeError."""
    assert "setcellmanager ok" in named_plugins
    for what in ("updateforces", "dostep", "neighbors"):
        line = next(ln for ln in named_plugins if ln.startswith(what + " "))
        assert line.startswith(what + " RuntimeError:"), line
        assert "CUDA device" in line, line
    assert "bad-args gpu SyntaxError" in named_plugins and "bad-args ref SyntaxError" in named_plugins

"""The LPMD-side binding, host side: lpmd2_gb300/lpmd_plugin/gbmd.cc compiled against the
reference's liblpmd headers and loaded through liblpmd's own PluginLoader (the reference's
sources, built by oracle/Makefile's `ref` target), in a process that has no GPU.

Checks that the plugin is an lpmd::Integrator reachable by dynamic_cast, that its keywords and
defaults are processed by Module::ProcessArguments, and that a keyword without a value raises
the reference's SyntaxError.  Skipped where the reference checkout or its build is absent.
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

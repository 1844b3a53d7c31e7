"""The reference-side binding that INTEGRATION.md shows (a C++ class
implementing the reference's BaseSimulation, NBodySimulation/base.h:8-38, by
forwarding every member to include/sph_gb300.h) compiles against the
reference's own base.h, links against libsph_gb300.so and runs (CPU only:
without a GPU, sph_create reports SPH_ERR_NO_DEVICE and every later call an
invalid argument, which the binding prints -- nothing crashes).

The reference's headers need the same two stand-ins the oracle's harness
uses (oracle/shim: vecmath.h's MSVC-only unions, render.h's OpenGL command
buffer); everything else comes from the reference tree."""
import os
import re
import subprocess

import pytest

import nbodysimulation_experiment_gb300 as pkg
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MAIN = r'''
#include "vecmath_sub.h"
#include "render_stub.h"
#include <vector>
#include <string>
#include <string.h>
#include <stdio.h>
#include <float.h>
#define FPL_IMPLEMENTATION
#define FPL_NO_AUDIO
#define FPL_NO_VIDEO
#define FPL_NO_WINDOW
#define FPL_NO_INPUT
#include <final_platform_layer.h>
#undef fplStaticAssert
#define fplStaticAssert(e)
#define strcpy_s(dst, n, src) strncpy(dst, src, n)
#include "gb300_demo.h"

int main() {
	GB300Simulation sim;
	BaseSimulation *demo = &sim;  // how DemoApplication holds it (app.h:125)
	demo->ResetStats();
	demo->SetGravity(Vec2f(0.0f, -10.0f));
	demo->AddPlane(Vec2f(0.0f, 1.0f), -2.8125f);
	demo->AddParticle(Vec2f(0.0f, 0.0f), Vec2f(0.0f, 0.0f));
	demo->Update(1.0f / 60.0f);
	const SPHParameters &p = demo->GetParams();
	SPHStatistics &st = demo->GetStats();
	printf("binding ran: particles %zu, kernel height %g, max neighbours %zu\n", demo->GetParticleCount(),
	       (double)p.kernelHeight, (size_t)st.maxParticleNeighborCount);
	return 0;
}
'''


def _binding_source():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    src = [b for b in blocks if "class GB300Simulation" in b]
    assert len(src) == 1, "INTEGRATION.md must show the binding once"
    return src[0]


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_binding_compiles_links_and_runs(tmp_path):
    pkg.build()
    (tmp_path / "gb300_demo.h").write_text(_binding_source())
    (tmp_path / "main.cpp").write_text(MAIN)
    ref = oracle.REFERENCE_TREE
    libdir = os.path.dirname(pkg.LIB_PATH)
    exe = str(tmp_path / "demo")
    cmd = ["g++", "-std=c++17", "-w", "-I" + str(tmp_path), "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ref, "NBodySimulation"),
           "-I" + os.path.join(ref, "include"), str(tmp_path / "main.cpp"), "-o", exe, "-L" + libdir,
           "-lsph_gb300", "-Wl,-rpath," + libdir, "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    assert "binding ran" in run.stdout

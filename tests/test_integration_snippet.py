"""The C++ binding of the GB300 step in the integration guide compiles
against the reference's own LBMSolver (src/lbm/solver.h, src/lbm/solver.cpp).

The code block of the guide's C++ section is compiled, with
``g++ -fsyntax-only``, in a translation unit that includes the reference's
solver the way the reference harness does (oracle/ref_harness.cpp: the
reference sources prepared by oracle/build_ref.sh, the serial MPI stub, the
class's private members opened, standing in for the one-line friend
declaration the binding asks the maintainer to add) and instantiates the
backend for every lattice and equation the reference's executor builds.
Skipped where the reference sources are not present (the GPU machine).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_OUT = os.path.join(ROOT, "oracle", "_ref")


def _snippet() -> str:
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("## C++ (the reference's own language)"):]
    m = re.search(r"```cpp\n(.*?)```", sec, flags=re.S)
    assert m, "no C++ block in the integration guide"
    return m.group(1)


def _reference_root():
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), "--root"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else None


TU = r"""
// the standard headers first, as the harness does: the access macro below
// must not reach them
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include <mpi.h>
// the friend declaration of the binding, emulated as the harness opens the class
#define private public
#define protected public
#include <sfcmm_common.h>
#include "config.h"
#include "lbm/solver.cpp"
#undef private
#undef protected

// ---- the integration guide's C++ section ----
%s
// ------------------------

template struct LBMGpuBackend<Debug_Level::no_debug, LBMethodType::D2Q9, LBEquationType::Navier_Stokes>;
template struct LBMGpuBackend<Debug_Level::no_debug, LBMethodType::D2Q9, LBEquationType::Poisson>;
template struct LBMGpuBackend<Debug_Level::no_debug, LBMethodType::D2Q5, LBEquationType::Poisson>;
template struct LBMGpuBackend<Debug_Level::no_debug, LBMethodType::D1Q3, LBEquationType::Poisson>;
"""


def test_integration_snippet_compiles_against_the_reference(tmp_path):
    ref = _reference_root()
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not ref or not os.path.isdir(os.path.join(ref, "src", "lbm")) or not os.path.exists(os.path.join(REF_OUT, "config.h")) \
            or not os.path.isdir(os.path.join(REF_OUT, "src")) or not cxx:
        pytest.skip("reference sources (oracle/build_ref.sh) or a C++ compiler not present")
    src = tmp_path / "integration_check.cpp"
    src.write_text(TU % _snippet())
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-fopenmp", "-w", "-I", os.path.join(ROOT, "oracle", "mpi_stub"), "-I", REF_OUT,
           "-I", os.path.join(REF_OUT, "src"), "-I", os.path.join(ref, "include"), "-isystem", os.path.join(ref, "external"),
           "-I", os.path.join(ROOT, "include"), str(src)]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-4000:]

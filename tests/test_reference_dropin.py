"""The drop-in boundary against the reference's own engine sources (CPU only).

Copies the reference's simulation/src into a temporary directory, applies the
patch to Physics/Simulation.h that the integration notes give (the drop-in
header in place of Tree/Tree.h and TimeIntegration.h, and Tree /
TimeIntegration as aliases of ag2host::Tree<Simulation> /
ag2host::TimeIntegration), drops Tree.cpp, Node.cpp and TimeIntegration.cpp
from the sources, and compiles and links the reference's executable
(main.cpp, Simulation.cpp with its call sites at :121-139 and :256-341,
DataManager, Log, Console, ...) against libag2.so.  The executable must link
with every Tree / TimeIntegration call resolved through the C-ABI.  It is not
run here: it needs a GPU, the reference's Config.ini and its input files.

Skipped where there is no reference checkout (AG2_REF, or the location
oracle/Makefile names).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle  # noqa: E402

REF = oracle.reference_checkout()

# Physics/Simulation.h of the reference: each line and what replaces it
PATCH = [
    ('#include "TimeIntegration.h"', '#include "ag2_tree.hpp"'),
    ('#include "Tree/Tree.h"', ''),
    ('class Tree;', 'class Simulation;\nusing Tree = ag2host::Tree<Simulation>;\n'
                    'using TimeIntegration = ag2host::TimeIntegration;'),
]
DROPPED = {os.path.join("Physics", "Tree", "Tree.cpp"), os.path.join("Physics", "Tree", "Node.cpp"),
           os.path.join("Physics", "TimeIntegration.cpp")}


def patch_simulation_header(text: str) -> str:
    lines = text.split("\n")
    for old, new in PATCH:
        hits = [k for k, l in enumerate(lines) if l.strip() == old]
        assert len(hits) == 1, f"expected one line '{old}' in Simulation.h, found {len(hits)}"
        lines[hits[0]] = new
    return "\n".join(lines)


@pytest.mark.skipif(REF is None, reason="no reference checkout")
def test_reference_engine_links_against_the_dropin(tmp_path):
    import build

    lib = build.build()
    src = tmp_path / "src"
    shutil.copytree(os.path.join(REF, "simulation", "src"), src)
    h = src / "Physics" / "Simulation.h"
    h.write_text(patch_simulation_header(h.read_text()))
    # the reference's CMakeLists.txt: src and its immediate subdirectories
    inc = ["-I" + str(src)] + ["-I" + str(src / d) for d in sorted(os.listdir(src)) if (src / d).is_dir()]
    inc += ["-I" + os.path.join(REPO, "include"), "-I" + os.path.join(REPO, "astrogenesis2.0_gb300", "host")]
    cpps = sorted(os.path.relpath(os.path.join(r, f), src) for r, _, fs in os.walk(src) for f in fs
                  if f.endswith(".cpp"))
    used = [c for c in cpps if c not in DROPPED]
    assert len(used) == len(cpps) - len(DROPPED)
    objs = tmp_path / "obj"
    objs.mkdir()

    def compile_one(rel):
        o = objs / (rel.replace(os.sep, "_") + ".o")
        r = subprocess.run(["g++", "-std=c++17", "-O0", "-fopenmp", "-w", *inc, "-c", str(src / rel), "-o", str(o)],
                           capture_output=True, text=True)
        assert r.returncode == 0, f"{rel} does not compile against the drop-in:\n{r.stderr[-3000:]}"
        return str(o)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        ofiles = list(ex.map(compile_one, used))
    exe = tmp_path / "AstroGen2"
    libdir = os.path.dirname(lib)
    r = subprocess.run(["g++", "-fopenmp", "-o", str(exe), *ofiles, "-L" + libdir, "-lag2",
                        "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, f"link failed:\n{r.stderr[-3000:]}"
    # the Tree / TimeIntegration work now goes through the C-ABI
    und = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    for sym in ("ag2_create", "ag2_upload", "ag2_build_tree", "ag2_sph_density", "ag2_forces",
                "ag2_visual_density", "ag2_root_radius"):
        assert sym in und, sym
    # and nothing of the reference's own tree remains
    defined = subprocess.run(["nm", "-C", "--defined-only", str(exe)], capture_output=True, text=True).stdout
    assert "Node::insert" not in defined and "Tree::buildTree" not in defined

"""The C ABI: the library loads without a GPU, exports every function that
include/*.h declares, and the ctypes mirrors have the C layouts (CPU only)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


def _declared_functions():
    names = set()
    for h in ("sfgpu.h", "starflood_compat.h"):
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return"):
                names.add(name)
    return sorted(names)


@pytest.fixture(scope="module")
def built_lib():
    from starflood_gb300 import build
    build.build()
    import starflood_gb300 as sf
    return sf.lib()


def test_exports_every_declared_symbol(built_lib):
    names = _declared_functions()
    assert "sfgpu_create" in names and "sim_step" in names and "tree_build" in names
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, missing


def test_struct_layouts_match_c(built_lib):
    import starflood_gb300 as sf
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "starflood_compat.h"
    int main(void) {
        printf("%zu %zu %zu %zu %zu %zu\n", sizeof(sfgpu_params), offsetof(sfgpu_params, flags),
               sizeof(node_t), sizeof(tree_t), sizeof(sim_t), offsetof(sim_t, tree));
        return 0;
    }
    """
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-std=c11", "-I" + INCLUDE, c, "-o", exe])
        out = [int(x) for x in subprocess.check_output([exe]).split()]
    assert out[0] == C.sizeof(sf.Params)
    assert out[1] == sf.Params.flags.offset
    assert out[2] == C.sizeof(sf.NodeT) == 80  # node_t of the FP32 reference (tree.h:16-25)
    assert out[3] == C.sizeof(sf.TreeT)
    assert out[4] == C.sizeof(sf.SimT)
    assert out[5] == sf.SimT.tree.offset


def test_defaults_are_reference_config(built_lib):
    import starflood_gb300 as sf
    p = sf.default_params()
    assert (p.dt, p.eps, p.G, p.theta) == (1.0, 1e-3, 1.0, 0.5)  # src/config.h
    assert (p.leaf_cap, p.depth_max, p.nodes_max) == (8, 16, 262144)
    assert p.solver == sf.SOLVER_TREE and p.sph == sf.SPH_OFF
    assert sf.dof(p) == 13 and sf.dof(sf.default_params(sph=sf.SPH_REFERENCE)) == 16


def test_reference_abi_sizes_when_available():
    """node_t / tree_t / sim_t of the compiled reference have the same sizes."""
    from oracle.build import REFERENCE_SRC as ref
    if not os.path.isdir(ref):
        pytest.skip("reference sources not present")
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "simulation.h"
    int main(void) { printf("%zu %zu %zu %zu\n", sizeof(node_t), sizeof(tree_t), sizeof(sim_t),
                            offsetof(sim_t, tree)); return 0; }
    """
    from oracle.build import reference_config, REF_VARIANTS
    with tempfile.TemporaryDirectory() as d:
        open(os.path.join(d, "config.h"), "w").write(reference_config(REF_VARIANTS["tree_e0.01"]))
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-std=c99", "-iquote", d, "-I-", "-I" + ref, c, "-o", exe],
                              stderr=subprocess.DEVNULL)
        out = [int(x) for x in subprocess.check_output([exe]).split()]
    import starflood_gb300 as sf
    assert out == [C.sizeof(sf.NodeT), C.sizeof(sf.TreeT), C.sizeof(sf.SimT), sf.SimT.tree.offset]


def test_fails_loudly_without_gpu(built_lib):
    import starflood_gb300 as sf
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(sf.SfgpuError):
        sf.Sim(16, sf.default_params(solver=sf.SOLVER_PP))


def test_rejects_empty_and_bad_parameters_before_the_device(built_lib):
    """N = 0 and out-of-range parameters fail in the host checks, with the
    library's message, before any CUDA call (so also on a machine without a
    GPU).  The reference's sim_init accepts N = 0 (malloc(0)) and its loops
    then do nothing; here an empty simulation is an error."""
    import starflood_gb300 as sf
    with pytest.raises(sf.SfgpuError, match="N must be > 0"):
        sf.Sim(0, sf.default_params(solver=sf.SOLVER_PP))
    with pytest.raises(sf.SfgpuError, match="eps must be > 0"):
        sf.Sim(16, sf.default_params(solver=sf.SOLVER_PP, eps=0.0))
    with pytest.raises(sf.SfgpuError, match="leaf_cap must be in"):
        sf.Sim(16, sf.default_params(solver=sf.SOLVER_TREE, leaf_cap=0))


def test_reference_main_links_against_library():
    """The drop-in at link time: the reference's
    own main.c, initcond.c, simulation_io.c and log.c, compiled from its
    sources with SOLVER_VIS off, link against libsfgpu.so in place of the
    solver objects, and every sim_* / vis_* symbol main.c needs resolves to
    the library."""
    from oracle.build import REFERENCE_SRC as ref, REF_VARIANTS, reference_config
    if not os.path.isfile(os.path.join(ref, "main.c")):
        pytest.skip("reference sources not present")
    import starflood_gb300 as sf
    libdir = os.path.dirname(sf.LIB_PATH)
    if not os.path.exists(sf.LIB_PATH):
        pytest.skip("libsfgpu.so not built")
    with tempfile.TemporaryDirectory() as d:
        open(os.path.join(d, "config.h"), "w").write(reference_config(REF_VARIANTS["tree_e0.01"]))
        objs = []
        for unit in ("main", "initcond", "simulation_io", "log"):
            o = os.path.join(d, unit + ".o")
            subprocess.check_call(["gcc", "-std=c99", "-O1", "-fopenmp", "-iquote", d, "-I-", "-I" + ref, "-c",
                                   os.path.join(ref, unit + ".c"), "-o", o], stderr=subprocess.DEVNULL)
            objs.append(o)
        exe = os.path.join(d, "starflood_gpu")
        subprocess.check_call(["gcc", "-fopenmp", *objs, "-L" + libdir, "-lsfgpu", "-Wl,-rpath," + libdir, "-lm",
                               "-o", exe])
        undef = subprocess.check_output(["nm", "-D", "--undefined-only", exe], text=True).split()
        exported = set(subprocess.check_output(["nm", "-D", "--defined-only", sf.LIB_PATH], text=True).split())
    wanted = [s for s in undef if s.startswith(("sim_", "tree_", "solve_", "vis_", "grid_"))]
    assert {"sim_init", "sim_free", "sim_solv", "sim_step", "sim_find"} <= set(wanted)
    assert all(s in exported for s in wanted), [s for s in wanted if s not in exported]

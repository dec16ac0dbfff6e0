"""Build recipe for the test oracle (TEST INFRASTRUCTURE ONLY).

Two products, both written only under ``oracle/``:

* ``oracle/liboracle_f32.so`` / ``liboracle_f64.so`` -- the C restatement in
  ``oracle/oracle.c`` (FP32 = the reference's arithmetic, FP64 = the FP64
  oracle).  Built everywhere, including the GPU host, with OpenMP so that the
  same library doubles as the timed CPU baseline.
* ``oracle/_ref/libref_<variant>.so`` -- the unmodified Starflood reference,
  compiled from its own sources where they lie (``REFERENCE_SRC``) against a
  generated ``config.h`` and linked with ``oracle/ref_harness.c``.  Only built
  when the reference tree is present; it is used to pin the restatement and to
  write the golden fixtures in ``tests/golden/``.

The reference's ``config.h`` #defines its parameters unconditionally, so a
``-D`` cannot override them; instead a patched copy is written to
``oracle/_ref/<variant>/config.h`` and found first through ``-iquote`` plus
``-I-`` (which stops GCC from searching the including file's own directory
first for quoted includes).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference sources: STARFLOOD_REFERENCE_SRC if set, else where this
# recipe expects the read-only Starflood tree.
REFERENCE_SRC = os.environ.get("STARFLOOD_REFERENCE_SRC", "/root/reference/src")
REF_OUT = os.path.join(HERE, "_ref")

CFLAGS = ["-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
          "-Wall", "-Wno-unused-result", "-Wno-unused-variable", "-Wno-unused-but-set-variable"]

# Reference configurations captured as golden fixtures.  Parameters follow the
# workloads they pin (PP eps=0.01 N=4096; BH theta=0.5; SPH h=0.05; PP
# eps=0.005 for the 1M-body Plummer case).
REF_VARIANTS = {
    "pp_e0.01": dict(tree=False, sph=False, fp64=False, eps="1.000e-2", dt="1.000e-3", theta="0.5"),
    "pp64_e0.01": dict(tree=False, sph=False, fp64=True, eps="1.000e-2", dt="1.000e-3", theta="0.5"),
    "pp_e0.005": dict(tree=False, sph=False, fp64=False, eps="5.000e-3", dt="1.000e-3", theta="0.5"),
    "tree_e0.01": dict(tree=True, sph=False, fp64=False, eps="1.000e-2", dt="1.000e-3", theta="0.5"),
    "tree_sph_e0.01": dict(tree=True, sph=True, fp64=False, eps="1.000e-2", dt="5.000e-4", theta="0.5"),
    "pp_sph_e0.01": dict(tree=False, sph=True, fp64=False, eps="1.000e-2", dt="5.000e-4", theta="0.5"),
}


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force: bool = False) -> list[str]:
    """Compile the C restatement twice (float and double)."""
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    outs = []
    jobs = []
    for tag, real, extra in (("f32", "float", []), ("f64", "double", ["-DORC_IS_DOUBLE"])):
        out = os.path.join(HERE, "liboracle_%s.so" % tag)
        outs.append(out)
        if force or not _newer(out, [src, hdr, __file__]):
            jobs.append(["gcc", *CFLAGS, "-shared", "-DORC_REAL=%s" % real, *extra,
                         "-o", out, src, "-lm"])
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return outs


def _set_macro(text: str, name: str, value: str | None) -> str:
    """Turn every '#define NAME ...' line (commented or not) into the wanted
    definition, or comment it out when value is None."""
    pat = re.compile(r"^[ \t]*(//)?[ \t]*#define[ \t]+%s\b.*$" % re.escape(name), re.M)
    if not pat.search(text):
        raise KeyError(name)
    repl = ("#define %s %s" % (name, value)).rstrip() if value is not None else "//#define %s" % name
    return pat.sub(lambda _m: repl, text)


def reference_config(variant: dict) -> str:
    with open(os.path.join(REFERENCE_SRC, "config.h")) as f:
        text = f.read()
    for off in ("SOLVER_VIS", "ENABLE_TIMING", "LOG_STATISTICS", "LOG_TIMINGS_SIM_STEP",
                "LOG_TIMINGS_VIS_DRAW", "LOG_TIMINGS_FFT_EXEC", "ENABLE_VIS_IO_THREAD",
                "ENABLE_STB_IMAGE_WRITE", "PAIRWISE_SOLVER_DECIMATION", "ENABLE_OFFLOAD_VIS"):
        text = _set_macro(text, off, None)
    text = _set_macro(text, "TIMESTEP_SIZE", variant["dt"])
    text = _set_macro(text, "EPSILON", variant["eps"])
    text = _set_macro(text, "TREE_THETA", variant["theta"])
    text = _set_macro(text, "G", "1.000")
    text = _set_macro(text, "ENABLE_TREE", "" if variant["tree"] else None)
    text = _set_macro(text, "ENABLE_SPH", "" if variant["sph"] else None)
    text = _set_macro(text, "STARFLOOD_DOUBLE_PRECISION", "" if variant["fp64"] else None)
    return text


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_SRC, "simulation.c"))


def build_reference(names: list[str] | None = None, force: bool = False) -> list[str]:
    """Compile the reference in place, one shared library per variant."""
    if not reference_available():
        return []
    names = list(REF_VARIANTS) if names is None else names
    harness = os.path.join(HERE, "ref_harness.c")
    outs = []
    jobs = []
    for name in names:
        v = REF_VARIANTS[name]
        cfg_dir = os.path.join(REF_OUT, name)
        os.makedirs(cfg_dir, exist_ok=True)
        cfg = os.path.join(cfg_dir, "config.h")
        text = reference_config(v)
        if not os.path.exists(cfg) or open(cfg).read() != text:
            with open(cfg, "w") as f:
                f.write(text)
        units = ["simulation", "gravity", "sph", "log", "grid"] + (["tree"] if v["tree"] else [])
        if not v["fp64"]:
            units += ["simulation_io", "visualization", "visualization_io", "initcond"]  # I/O, vis, ICs
        srcs = [os.path.join(REFERENCE_SRC, u + ".c") for u in units]
        out = os.path.join(REF_OUT, "libref_%s.so" % name)
        outs.append(out)
        if force or not _newer(out, srcs + [harness, cfg, __file__]):
            jobs.append(["gcc", *CFLAGS, "-shared", "-iquote", cfg_dir, "-I-",
                         "-I" + REFERENCE_SRC, "-o", out, *srcs, harness, "-lm"])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    return outs


def build(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force=force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built:", os.listdir(HERE))

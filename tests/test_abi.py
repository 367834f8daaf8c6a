"""The C-ABI library loads on a host without a GPU, exports every function
include/*.h declares, and its struct layouts match the Python binding."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(exa_[a-z0-9_]+)\s*\(", src)))


def exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_exastitch_exports_all_declared(native):
    from owlexastitcher_gb300 import exastitch as E
    lib = os.path.join(ROOT, "owlexastitcher_gb300", "libexastitch.so")
    names = declared("exastitch.h")
    assert len(names) >= 20
    missing = [n for n in names if n not in exported(lib)]
    assert not missing, missing
    assert set(E.EXPORTED) <= set(names)
    E.lib()  # loads and checks the struct layouts


def test_generator_exports_all_declared(native):
    lib = os.path.join(ROOT, "owlexastitcher_gb300", "libexagen.so")
    names = declared("exastitch_gen.h")
    missing = [n for n in names if n not in exported(lib)]
    assert not missing, missing


def test_abi_sizes(native):
    from owlexastitcher_gb300 import exastitch as E
    L = E.lib()
    assert L.exa_abi_sizeof(0) == E.C.sizeof(E.LaunchParams)
    assert L.exa_abi_sizeof(1) == 32 and L.exa_abi_sizeof(2) == 12
    assert L.exa_abi_sizeof(12) == E.C.sizeof(E.RenderStats) and L.exa_abi_sizeof(13) == E.C.sizeof(E.BuildStats)
    assert L.exa_abi_sizeof(14) == E.BRICK_DTYPE.itemsize and L.exa_abi_sizeof(15) == E.ABR_DTYPE.itemsize
    assert L.exa_abi_sizeof(16) == 0
    assert L.exa_sampler_class_name() == b"ExaStitchSampler"


def test_launch_params_defaults(native):
    from owlexastitcher_gb300 import exastitch as E
    lp = E.new_launch_params()
    assert lp.integrator == E.PATH_TRACING_INTEGRATOR and lp.render.spp == 1
    assert lp.ext.maxBounces == 1024 and lp.ext.albedo < 0 and lp.ext.hgG == 0.0
    assert lp.voxelSpaceTransform.l.vx.x == 1.0 and lp.transferFunc.opacityScale == 1.0


def test_calls_without_context_fail_cleanly(native):
    from owlexastitcher_gb300 import exastitch as E
    L = E.lib()
    assert L.exa_sampler_build(None) == E.EXA_ERR_STATE
    assert b"no model" in L.exa_last_error()
    assert L.exa_render(None, None, 1, 1) == E.EXA_ERR_STATE


def test_python_constants_match_header():
    """every integer constant of include/exastitch.h that the Python binding
    mirrors (as EXA_NAME or NAME) has the header's value"""
    from owlexastitcher_gb300 import exastitch as E
    src = open(os.path.join(ROOT, "include", "exastitch.h")).read()
    defs = {}
    for name, body in re.findall(r"#define\s+(EXA_[A-Z0-9_]+)[ \t]+([^\n/]+)", src):
        body = body.strip()
        m = re.fullmatch(r"\(?\s*(-?(?:0x[0-9a-fA-F]+|\d+))u?\s*\)?", body)
        s = re.fullmatch(r"\(\s*(\d+)u?\s*<<\s*(\d+)\s*\)", body)
        if m:
            defs[name] = int(m.group(1), 0)
        elif s:
            defs[name] = int(s.group(1)) << int(s.group(2))
    matched = 0
    for name, value in defs.items():
        for py in (name, name[4:]):
            if hasattr(E, py):
                assert getattr(E, py) == value, (name, getattr(E, py), value)
                matched += 1
                break
    assert matched >= 25, matched

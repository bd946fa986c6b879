"""The N-API addon (webgpu-bcmc_gb300/node/bcmc_node.cc) compiled as host C++
against a stand-in node_api.h that holds Node-API's documented declarations
(tests/host_device/napi/), since Node.js and its headers are absent here: the
addon compiles with warnings as errors, every C-ABI entry point it calls is
declared in include/bcmc.h and exported by the built library, and it registers
the reference's method names (js/compressed_marching_cubes.js:432,580,366)."""
import os
import re
import shutil
import subprocess

import pytest

from bcmc import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ADDON = os.path.join(ROOT, "webgpu-bcmc_gb300", "node", "bcmc_node.cc")
BUILD = os.path.join(HERE, "_build")


@pytest.fixture(scope="module")
def addon_object():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    os.makedirs(BUILD, exist_ok=True)
    obj = os.path.join(BUILD, "bcmc_node.o")
    cmd = [cxx, "-std=c++17", "-O1", "-fPIC", "-c", "-Wall", "-Wextra", "-Werror", "-DNODE_GYP_MODULE_NAME=bcmc_node",
           "-I", os.path.join(HERE, "host_device", "napi"), "-I", os.path.join(ROOT, "include"), ADDON, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return obj


def _undefined(obj):
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("no nm")
    r = subprocess.run([nm, "-u", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return sorted({line.split()[-1] for line in r.stdout.splitlines() if line.strip()})


def test_addon_calls_only_exported_entry_points(addon_object, lib_built):
    und = _undefined(addon_object)
    bcmc = [s for s in und if s.startswith("bcmc_")]
    assert len(bcmc) >= 8, bcmc
    L = _lib.load()
    missing = [s for s in bcmc if not hasattr(L, s)]
    assert not missing, missing
    assert set(bcmc) <= set(_lib.SIGNATURES)
    # the GPU is reached through the C ABI alone: no CUDA runtime or driver call
    direct = [s for s in und if s.startswith(("cuda", "cu", "nccl"))]
    assert not direct, direct


def test_addon_registers_the_reference_method_names(addon_object):
    src = open(ADDON).read()
    init = src[src.index("napi_value Init("):]
    names = set(re.findall(r'\{"([A-Za-z]+)",\s*nullptr,', init))
    assert {"setCompressedVolume", "computeSurface", "reportMemoryUse"} <= names, names
    assert '"CompressedMarchingCubes"' in init
    # the entry point Node.js looks up is defined by the module registration
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("no nm")
    r = subprocess.run([nm, "--defined-only", addon_object], capture_output=True, text=True)
    assert "napi_register_module_v1" in r.stdout

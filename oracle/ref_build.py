"""Builds oracle/_ref/libbcmc_ref.so: the reference's own compute shaders
compiled as host C++ (TEST INFRASTRUCTURE ONLY).

The reference (Twinklebear/webgpu-bcmc) runs its pipeline as GLSL compute
shaders under WebGPU, which cannot run here.  GLSL 4.50 compute code is close
to C++, so this recipe reads the shader files where they lie in the reference
checkout, applies a fixed list of mechanical rewrites (below), and compiles each
program with oracle/ref_shim.h (vector types, built-ins, barrier) and
oracle/ref_runtime.cpp (workgroups as fibers).  Nothing of the reference is
copied into the repository: the rewritten sources are written to oracle/_ref/
(git-ignored) and compiled there.

The rewrites (no semantic edits to the shader bodies):
  * strip comments, `#version`, `layout(local_size_*) in;`
  * inline `#include "x.comp"` (the C preprocessor keeps include guards)
  * `layout(...) [readonly] buffer|uniform Name { members } [inst];` -> namespace-scope
    variables (runtime-sized arrays become pointers the harness binds)
  * `shared T x[N];` -> namespace-scope array (one workgroup runs at a time)
  * declarations without an initialiser get `{}` (WGSL zero-initialises
    function-scope variables)
  * GLSL array types `T[N] name` / `T[N][M] name` -> C declarators, and a
    function returning `float[8]` -> std::array<float, 8>
  * parameter qualifiers: `inout T x` -> `T& x`, `in T x` -> `T x`
    (array parameters are pointers in C++, which is `inout`)
  * float literals get an `f` suffix (GLSL literals are 32-bit)
  * swizzles `.xyz/.xy/.xz/.yz` -> glsl::swz_* helpers (`v.xyz = e` -> glsl::set_xyz)
  * vertex-stage `layout(location = n) in/out T x;` -> namespace-scope variables
  * `.rgb` -> `.xyz`, `.a` -> `.w`, `v.xyz += e` -> `v.xyz = v.xyz + (e)`
  * min/max/abs/ldexp/ceil and the geometric/exponential built-ins and
    dFdx/dFdy -> glsl_* helpers, barrier() -> ref_barrier(), main -> main_
  * compiled with the defines shaders/embed_shaders.py passes (BLOCK_SIZE=512,
    SORT_CHUNK_SIZE=64), and DRAW_FOG for the fog variants of the render shaders
  * every program lives in its own namespace and translation unit

Usage: python oracle/ref_build.py [--reference DIR]
(default DIR: $BCMC_REFERENCE, else a checkout named `reference` beside this
repository's folder).  Exits 0 with a message and builds nothing when the
reference checkout is absent.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB = os.path.join(OUT, "libbcmc_ref.so")

# shader program -> namespace
PROGRAMS = {
    "zfp_decompress_block": "zfp_decompress_block.comp",
    "zfp_compute_block_range": "zfp_compute_block_range.comp",
    "compute_block_active": "compute_block_active.comp",
    "compute_block_has_vertices": "compute_block_has_vertices.comp",
    "compute_block_voxel_num_verts": "compute_block_voxel_num_verts.comp",
    "compute_block_vertices": "compute_block_vertices.comp",
    # the render pass's shaders: the vertex stage's position math, with DRAW_FOG
    # also the fog entry distance, and the fragment shading with and without fog
    "mc_isosurface_vert": "mc_isosurface.vert",
    "mc_isosurface_vert_fog": "mc_isosurface.vert",
    "mc_isosurface_frag": "mc_isosurface.frag",
    "mc_isosurface_frag_fog": "mc_isosurface.frag",
    # RadixSorter (js/radix_sort_by_key.js): chunk sort, merges, reverse
    "radix_sort_chunk": "radix_sort_chunk.comp",
    "merge_sorted_chunks": "merge_sorted_chunks.comp",
    "reverse_buffer": "reverse_buffer.comp",
    # LRUCache (js/lru_cache.js): age, mark, extract, init, sort-key copy, assignment
    "lru_cache_age_slots": "lru_cache_age_slots.comp",
    "lru_cache_mark_new_items": "lru_cache_mark_new_items.comp",
    "lru_cache_extract_slot_available": "lru_cache_extract_slot_available.comp",
    "lru_cache_init": "lru_cache_init.comp",
    "lru_copy_available_slot_age": "lru_copy_available_slot_age.comp",
    "lru_cache_update": "lru_cache_update.comp",
    # ExclusiveScanner (js/exclusive_scan.js): block scan, scan of the block sums, add-back
    "prefix_sum": "prefix_sum.comp",
    "block_prefix_sum": "block_prefix_sum.comp",
    "add_block_sums": "add_block_sums.comp",
    # StreamCompact (js/stream_compact.js)
    "stream_compact": "stream_compact.comp",
}
# what shaders/embed_shaders.py passes to every shader compile
DEFINES = ["-DBLOCK_SIZE=512", "-DSORT_CHUNK_SIZE=64"]
# per-program defines (js/bcmc.js builds the fog variant of the render pipeline with DRAW_FOG)
PROGRAM_DEFINES = {"mc_isosurface_vert_fog": ["DRAW_FOG"], "mc_isosurface_frag_fog": ["DRAW_FOG"]}


def reference_dir(arg: str | None) -> str:
    beside = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return arg or os.environ.get("BCMC_REFERENCE") or beside


def strip_comments(s: str) -> str:
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", "", s)


def inline_includes(path: str, seen=None) -> str:
    seen = set() if seen is None else seen
    text = strip_comments(open(path).read())
    base = os.path.dirname(path)

    def rep(m):
        inc = os.path.join(base, m.group(1))
        return inline_includes(inc, seen)

    return re.sub(r'#include\s+"([^"]+)"', rep, text)


def convert_blocks(s: str) -> str:
    """layout(...) buffer/uniform Name { members } [instance];"""

    def rep(m):
        out = []
        for decl in m.group(3).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            rt = re.fullmatch(r"(\w+)\s+(\w+)\s*\[\s*\]", decl)
            if rt:  # runtime-sized array: bound by the harness
                out.append(f"{rt.group(1)}* {rt.group(2)} = nullptr;")
            else:
                out.append(f"{decl} {{}};" if "[" in decl else f"{decl} {{}};")
        return "\n".join(out) + "\n"

    return re.sub(r"layout\s*\([^)]*\)\s*(?:(?:readonly|writeonly|coherent|restrict)\s+)*(buffer|uniform)\s+(\w+)"
                  r"\s*\{(.*?)\}\s*\w*\s*;", rep, s, flags=re.S)


def transform(text: str) -> str:
    s = text
    s = re.sub(r"#version[^\n]*\n", "\n", s)
    s = re.sub(r"layout\s*\(\s*local_size[^)]*\)\s*in\s*;", "", s)
    s = convert_blocks(s)
    # vertex-stage inputs/outputs: namespace-scope variables the harness sets/reads
    s = re.sub(r"layout\s*\(\s*location\s*=\s*\d+\s*\)\s*(in|out)\s+(\w+)\s+(\w+)\s*;", r"\2 \3{};", s)
    s = re.sub(r"\bshared\s+", "", s)
    # arrays returned by value
    s = re.sub(r"\bfloat\s*\[\s*8\s*\]\s+(\w+)\s*\(", r"std::array<float, 8> \1(", s)
    s = re.sub(r"\bfloat\s+values\s*\[\s*8\s*\]\s*;", "std::array<float, 8> values;", s)
    s = re.sub(r"\b(const\s+)?float\s+(\w+)\s*\[\s*8\s*\]\s*=\s*compute_vertex_values\(",
               r"\1std::array<float, 8> \2 = compute_vertex_values(", s)
    # GLSL array types -> C declarators
    s = re.sub(r"\b(const\s+)?(\w+)\s*\[\s*([^\]\[]+?)\s*\]\s*\[\s*([^\]\[]+?)\s*\]\s+(\w+)\s*=",
               r"\1\2 \5[\3][\4] =", s)
    s = re.sub(r"\b(const\s+)?(\w+)\s*\[\s*([^\]\[]+?)\s*\]\s+(\w+)\s*=", r"\1\2 \4[\3] =", s)
    # WGSL zero-initialises function-scope variables: give every declaration
    # without an initialiser one (`T x;` -> `T x{};`, `T x[N];` -> `T x[N] = {};`)
    s = re.sub(r"(?m)^(\s*)(?!return\b|else\b|case\b|goto\b)(\w+)\s+(\w+)\s*(\[[^\]]*\])\s*;\s*$",
               r"\1\2 \3\4 = {};", s)
    s = re.sub(r"(?m)^(\s*)(?!return\b|else\b|case\b|goto\b)(\w+)\s+(\w+)\s*;\s*$", r"\1\2 \3{};", s)
    # parameter qualifiers
    s = re.sub(r"\binout\s+(\w+)\s+(\w+)\s*\[", r"\1 \2[", s)
    s = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", s)
    s = re.sub(r"([(,]\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", s)
    s = re.sub(r"([(,]\s*)out\s+(\w+)\s+(\w+)", r"\1\2& \3", s)
    # 32-bit float literals
    s = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])",
               r"\1f", s)
    # swizzles and built-ins (.rgb/.a are .xyz/.w; `v.xyz += e` assigns v.xyz + e)
    s = re.sub(r"\.rgb\b", ".xyz", s)
    s = re.sub(r"\b(\w+)\.a\b", r"\1.w", s)
    s = re.sub(r"\b(\w+)\.xyz\s*\+=\s*([^;]+);", r"glsl::set_xyz(\1) = glsl::swz_xyz(\1) + (\2);", s)
    s = re.sub(r"\b(\w+)\.xyz\s*=(?!=)", r"glsl::set_xyz(\1) =", s)
    s = re.sub(r"\b(\w+)\.(xyz|xy|xz|yz)\b", r"glsl::swz_\2(\1)", s)
    s = re.sub(r"\b(min|max|abs|ldexp|ceil|dot|length|normalize|cross|clamp|pow|exp|dFdx|dFdy)\s*\(",
               r"glsl_\1(", s)
    s = re.sub(r"\bbarrier\s*\(\s*\)", "ref_barrier()", s)
    s = re.sub(r"\bvoid\s+main\s*\(\s*(void)?\s*\)", "void main_()", s)
    return s


def tri_table_inc(ref: str) -> str:
    js = open(os.path.join(ref, "js", "tri_table.js")).read()
    body = js[js.index("[") + 1: js.rindex("]")]
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(vals) == 256 * 16, len(vals)
    rows = [", ".join(str(v) for v in vals[i: i + 16]) for i in range(0, len(vals), 16)]
    return "static const int32_t kRefTriTable[4096] = {\n" + ",\n".join(rows) + "\n};\n"


def generate(ref: str) -> list:
    os.makedirs(GEN, exist_ok=True)
    shaders = os.path.join(ref, "shaders")
    with open(os.path.join(GEN, "tri_table.inc"), "w") as f:
        f.write("// generated from js/tri_table.js of the reference checkout\n" + tri_table_inc(ref))
    srcs = []
    for ns, fname in PROGRAMS.items():
        text = transform(inline_includes(os.path.join(shaders, fname)))
        path = os.path.join(GEN, f"{ns}.cpp")
        with open(path, "w") as f:
            f.write(f"// generated from shaders/{fname} of the reference checkout by oracle/ref_build.py\n")
            f.write('#include "ref_shim.h"\n#undef UINT_MAX\n')
            for d in PROGRAM_DEFINES.get(ns, []):
                f.write(f"#define {d} 1\n")
            f.write(f"namespace p_{ns} {{\n{text}\n}}  // namespace p_{ns}\n")
            f.write(f'#define REF_PROGRAM_{ns} 1\n#include "tri_table.inc"\n#include "ref_glue.inc"\n')
        srcs.append(path)
    return srcs


def build(ref: str | None = None, force: bool = False) -> str | None:
    ref = reference_dir(ref)
    if not os.path.isdir(os.path.join(ref, "shaders")):
        print(f"reference checkout not found at {ref}: oracle/_ref not built")
        return None
    deps = [os.path.join(HERE, f) for f in ("ref_shim.h", "ref_runtime.cpp", "ref_glue.inc", "ref_build.py")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    srcs = generate(ref) + [os.path.join(HERE, "ref_runtime.cpp")]
    flags = ["g++", "-std=c++20", "-O2", "-fPIC", "-fwrapv", "-ffp-contract=off", "-fno-fast-math",
             "-I", HERE, "-I", GEN] + DEFINES
    objs = []

    def cc(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        r = subprocess.run(flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(cc, srcs))
    subprocess.run(["g++", "-shared", "-o", LIB] + objs, check=True)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    lib = build(a.reference, a.force)
    print(lib or "not built")


if __name__ == "__main__":
    sys.exit(main())

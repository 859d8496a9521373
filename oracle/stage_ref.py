#!/usr/bin/env python3
"""Stage and patch the reference's CPU solver sources for the oracle build.

ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product path reads, links or
runs what this script produces.

It copies the reference's own ``src/*.cpp`` and ``include/*.h`` (the
morris821028/hw-radiosity tree, given by ``--ref``) into ``oracle/_ref/src/``
(git-ignored: reference sources are never committed) and applies a minimal,
behaviour-preserving patch set so the binary can be used as a checker:

1. ``shade.cpp:570``  ``*S.rbegin()`` on an empty set is undefined behaviour
   (it segfaults whenever no non-light triangle has area >= 1); guard it with
   ``if (S.empty()) break;`` which is what the loop does one line later anyway.
2. ``rad.h:10-11``    raise the static capacities ``MaxTriList`` and
   ``MaxTreeNode``.  Capacities only: ``MaxLevel`` and ``MaxTriPerNode`` (which
   define the octree) are untouched.  ``MaxTreeNode`` >= (8^7-1)/7 = 299,593
   covers every tree ``MaxLevel 6`` can produce.
3. ``rad.cpp:407``    one hook call per shooter step, ``rad_hook_shot(C)``
   (oracle/ref_hooks.cpp): shooter trace, per-step timestamps and an optional
   step limit.  The per-slot state dump runs from an ``atexit`` handler there.
4. ``raycast.cpp``    counter macros (rays, cells, triangle tests, edge-plane
   tests, "Precision Exceeded" re-steps) that compile to nothing unless
   ``RAD_COUNTERS`` is defined.

A third copy, ``oracle/_ref/src_adapt/``, replaces ``include/config.h`` by
ADAPT + ROLLBACK only: the adaptive split variant (serial loop, delta-FF split
test, no pre-partition).

``--fp64`` additionally rewrites ``float`` to ``double`` in the solver's data
types and arithmetic (vector.h, rad.h, shade.cpp, raycast.cpp and the rad.cpp
locals), keeping the command-line option globals as ``float`` and formatting
output through ``float``, to give the FP64 CPU build of the reference's own
algorithm.  It is staged into ``oracle/_ref/src64/``.
"""
import argparse
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _sub_once(text, old, new, what):
    n = text.count(old)
    if n != 1:
        raise SystemExit(f"stage_ref: anchor for '{what}' found {n} times")
    return text.replace(old, new)


def _patch_common(files):
    sh = files["src/shade.cpp"]
    sh = _sub_once(sh, "\t\tpair<float, int> t = *S.rbegin();",
                   "\t\tif (S.empty()) break;\n\t\tpair<float, int> t = *S.rbegin();",
                   "PrePartition empty-set guard")
    files["src/shade.cpp"] = sh

    rh = files["include/rad.h"]
    rh = _sub_once(rh, "#define MaxTriList\t200000", "#define MaxTriList\t64000000", "MaxTriList")
    rh = _sub_once(rh, "#define MaxTreeNode\t20000", "#define MaxTreeNode\t300000", "MaxTreeNode")
    files["include/rad.h"] = rh

    rc = files["src/rad.cpp"]
    rc = _sub_once(rc, "static int parallelRadiosity() {",
                   "bool rad_hook_shot(const vector<int>&);\nstatic int parallelRadiosity() {",
                   "hook prototype")
    rc = _sub_once(rc, "\tvector<int> C(listCanditate());\n",
                   "\tvector<int> C(listCanditate());\n\tif (rad_hook_shot(C)) return 0;\n",
                   "hook call")
    rc = _sub_once(rc, "\tphysrc = MaxDeltaRad();\n",
                   "\tphysrc = MaxDeltaRad();\n\t{ vector<int> C_; if (physrc >= 0) C_.push_back(physrc);"
                   " if (rad_hook_shot(C_)) return 0; }\n",
                   "serial hook call")
    files["src/rad.cpp"] = rc

    ry = files["src/raycast.cpp"]
    ry = _sub_once(ry, "\tCopyVector(p, q);\n\twhile ((currIdx = TreeNodeNum(q)) >= 0) {",
                   "\tCopyVector(p, q);\n\tRAD_CNT_RAY();\n\twhile ((currIdx = TreeNodeNum(q)) >= 0) {\n\t\tRAD_CNT_CELL();",
                   "ray/cell counters")
    ry = _sub_once(ry, "\ta1 = InnerProd(v, tp->n);", "\tRAD_CNT_TRI();\n\ta1 = InnerProd(v, tp->n);",
                   "triangle-test counter")
    ry = _sub_once(ry, "\tif (t >= *t_min)\n\t\treturn false;\n",
                   "\tif (t >= *t_min)\n\t\treturn false;\n\tRAD_CNT_SE();\n", "edge-test counter")
    ry = _sub_once(ry, "\t\t\tt += 1.0;\n", "\t\t\tRAD_CNT_PREC();\n\t\t\tt += 1.0;\n",
                   "precision counter")
    files["src/raycast.cpp"] = ry
    return files


def _to_fp64(files):
    """float -> double for the solver's state and arithmetic."""
    out = dict(files)
    vh = out["include/vector.h"]
    vh = vh.replace("typedef float\tVector[3];", "typedef double\tVector[3];")
    vh = vh.replace("typedef float\t*VectorPtr;", "typedef double\t*VectorPtr;")
    vh = vh.replace("typedef float \tMatrix[4][4];", "typedef double \tMatrix[4][4];")
    vh = vh.replace('fscanf(fp,"%f%f%f"', 'fscanf(fp,"%lf%lf%lf"')
    vh = vh.replace("inline float norm(", "inline double norm(")
    vh = vh.replace("inline float norm2(", "inline double norm2(")
    vh = vh.replace("\tfloat t = norm(p);", "\tdouble t = norm(p);")
    out["include/vector.h"] = vh

    rh = out["include/rad.h"]
    rh = rh.replace("#define ffabs(x) (float)fabs((double)(x))", "#define ffabs(x) fabs((double)(x))")
    rh = rh.replace("\tfloat   se[3][4];", "\tdouble  se[3][4];")
    rh = rh.replace("\tfloat\tarea;", "\tdouble\tarea;")
    out["include/rad.h"] = rh

    for name in ("src/shade.cpp", "src/raycast.cpp"):
        s = out[name]
        s = re.sub(r"\bfloat\b", "double", s)
        s = s.replace("pair<double, int>", "pair<double, int>")
        out[name] = s

    rc = out["src/rad.cpp"]
    # solver locals and accumulators; the option globals stay float
    rc = rc.replace("\tfloat m;\n", "\tdouble m;\n")
    rc = rc.replace("\tfloat minarea = 100000000.0, maxarea = 0.0;", "\tdouble minarea = 100000000.0, maxarea = 0.0;")
    rc = rc.replace("\t\tfloat scale = LightScale;", "\t\tdouble scale = LightScale;")
    rc = rc.replace("\t\tfloat maxDelta = 0.f;", "\t\tdouble maxDelta = 0.f;")
    rc = rc.replace("\t\t\tfloat delta = tp->deltaB[0] + tp->deltaB[1] + tp->deltaB[2];",
                    "\t\t\tdouble delta = tp->deltaB[0] + tp->deltaB[1] + tp->deltaB[2];")
    rc = rc.replace("\t\tfloat delta = tp->deltaB[0] + tp->deltaB[1] + tp->deltaB[2];",
                    "\t\tdouble delta = tp->deltaB[0] + tp->deltaB[1] + tp->deltaB[2];")
    rc = rc.replace("vector< pair<float, int> > C;", "vector< pair<double, int> > C;")
    rc = rc.replace("\t\t\tfloat f = 0;", "\t\t\tdouble f = 0;")
    rc = rc.replace("f = max(min(f, 255.0f), 0.0f);", "f = max(min(f, 255.0), 0.0);")
    rc = rc.replace("fp::tostring<float> z(tp->n[0]);", "fp::tostring<float> z((float)tp->n[0]);")
    rc = rc.replace("fp::tostring<float> z(tp->n[1]);", "fp::tostring<float> z((float)tp->n[1]);")
    rc = rc.replace("fp::tostring<float> z(tp->n[2]);", "fp::tostring<float> z((float)tp->n[2]);")
    rc = rc.replace("fp::tostring<float> z(tp->p[j][0]);", "fp::tostring<float> z((float)tp->p[j][0]);")
    rc = rc.replace("fp::tostring<float> z(tp->p[j][1]);", "fp::tostring<float> z((float)tp->p[j][1]);")
    rc = rc.replace("fp::tostring<float> z(tp->p[j][2]);", "fp::tostring<float> z((float)tp->p[j][2]);")
    out["src/rad.cpp"] = rc
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference tree (default: $RAD_REFERENCE_DIR, baseline/_ref, /root/reference)")
    ap.add_argument("--out", default=os.path.join(HERE, "_ref"))
    args = ap.parse_args()
    if args.ref is None:
        from runner import reference_dir
        args.ref = reference_dir() or "(none found)"
    if not os.path.isdir(os.path.join(args.ref, "src")):
        print(f"stage_ref: no reference tree at {args.ref}; nothing staged", file=sys.stderr)
        return 1
    names = ["src/rad.cpp", "src/shade.cpp", "src/raycast.cpp",
             "include/config.h", "include/rad.h", "include/vector.h",
             "include/raycast.h", "include/shade.h", "include/float2string.h"]
    files = {}
    for n in names:
        with open(os.path.join(args.ref, n)) as f:
            files[n] = f.read()
    files = _patch_common(files)
    # the adaptive split variant: include/config.h with ADAPT and ROLLBACK only
    # (serialRadiosity, the full Shade with its delta-FF split test, no
    # pre-partition) -- the configuration in which the split path is live
    adapt = dict(files)
    adapt["include/config.h"] = ("#ifndef _CONFIG_H\n#define _CONFIG_H\n"
                                 "#define ADAPT\n#define ROLLBACK\n#endif\n")
    for sub, fs in (("src", files), ("src64", _to_fp64(files)), ("src_adapt", adapt)):
        root = os.path.join(args.out, sub)
        if os.path.isdir(root):
            shutil.rmtree(root)
        for n, text in fs.items():
            p = os.path.join(root, n)
            os.makedirs(os.path.dirname(p), exist_ok=True)
            with open(p, "w") as f:
                f.write(text)
    # the result viewer's shaders, made compilable as C++ against
    # oracle/glsl_shim.h: the #extension and precision lines dropped and the
    # swizzles .xyz .rgb .a .s .t written as calls; nothing else changes
    lib = os.path.join(args.ref, "WebGL_demo", "public", "lib")
    if os.path.isdir(lib):
        out = os.path.join(args.out, "src_shaders")
        os.makedirs(out, exist_ok=True)
        for name in ("gouraud.vs", "flat.vs", "flat.fs"):
            with open(os.path.join(lib, name)) as f:
                lines = f.read().splitlines()
            kept = [ln for ln in lines if not re.match(r"\s*(#extension|precision)\b", ln)]
            text = re.sub(r"\.(xyz|rgb|a|s|t)\b", r".\1()", "\n".join(kept) + "\n")
            with open(os.path.join(out, name), "w") as f:
                f.write(text)
    # the result viewer's model converter (one file, unpatched): pins the
    # converter half of the headless renderer's input preparation
    conv = os.path.join(args.ref, "WebGL_demo", "model-converter", "main.cpp")
    if os.path.exists(conv):
        os.makedirs(os.path.join(args.out, "src_conv"), exist_ok=True)
        shutil.copyfile(conv, os.path.join(args.out, "src_conv", "main.cpp"))
    print(f"stage_ref: staged patched reference into {args.out}/src and src64")
    return 0


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python3
"""Generate a single-translation-unit build of the reference effmass sources.

This is test infrastructure for the oracle, not part of the product.  It
reads the reference C++23-module sources where they lie (read-only) and
writes ``oracle/_ref/ref_all.cpp`` (git-ignored).  The transforms are purely
mechanical so that GCC 13 (no ``import std``, no ``<print>``) can compile the
reference's own arithmetic:

* ``module;`` / ``export module X;`` / ``module X;`` / ``import ...;`` lines are
  dropped; files are concatenated in module-dependency order;
* ``export { ... }`` wrappers are unwrapped (contents kept) and a leading
  ``export`` keyword is removed;
* ``#include "pocketfft.h"`` / ``"pugixml.hpp"`` / ``"../physical_constants.hpp"``
  are replaced by the project-written shims in ``oracle/ref_shims.hpp``;
* the pugixml-based body of the UPF reader is cut (the class definition is
  kept); ``oracle/ref_driver.cpp`` defines ``UPF::UPF`` from an in-memory
  registry instead;
* ``private:`` sections of the β(q) table classes are opened so that the
  driver can export the raw tables the GPU path consumes.

Usage: python oracle/refgen.py REFERENCE_ROOT   (or EFFMASS_REFERENCE in the environment)
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")

# Dependency order of the reference modules (leaves first).
ORDER = [
    "src/utils/array2d.cppm",
    "src/utils/vector3d.cppm",
    "src/utils/logger.cppm",
    "src/io/lattice.cppm",
    "src/io/GKK.cppm",
    "src/io/WG.cppm",
    "src/io/RHO.cppm",
    "src/io/VR.cppm",
    "src/io/ATOM.cppm",
    "src/io/EIGEN.cppm",
    "src/io/OCC.cppm",
    "src/math/sph_bessel.cppm",
    "src/math/numerical.cppm",
    "src/math/fourier_bessel.cppm",
    "src/math/linalg.cppm",
    "src/math/sph_harmonics.cppm",
    "src/math/fft.cppm",
    "src/pseudo/io/upf.cppm",
    "src/pseudo/ncpp.cppm",
    "src/pseudo/ncpp_advance.cppm",
    "src/support/density.cppm",
    "src/H_psi/structure_factor.cppm",
    "src/H_psi/hamiltonian.cppm",
    "src/H_psi/hamiltonian.cpp",
    "src/H_psi/hamiltonian_callable.cpp",
    "src/H_psi/hamiltonian_gradient.cpp",
    "src/H_psi/hamiltonian_hessian.cpp",
]

DROP_INCLUDES = ("pocketfft.h", "pugixml.hpp", "physical_constants.hpp")


def unwrap_export_blocks(lines):
    """Remove `export {` and its matching `}` while keeping the contents."""
    out = []
    depth_stack = []  # brace depth at which an export block was opened
    depth = 0
    for line in lines:
        stripped = line.strip()
        if re.match(r"^export\s*\{\s*$", stripped):
            depth_stack.append(depth)
            depth += 1
            out.append("")
            continue
        opens = line.count("{")
        closes = line.count("}")
        if depth_stack and re.match(r"^\}\s*(//.*)?$", stripped) and depth - 1 == depth_stack[-1]:
            depth_stack.pop()
            depth -= 1
            out.append("")
            continue
        depth += opens - closes
        out.append(line)
    return out


def transform(path, text):
    lines = text.splitlines()
    out = []
    for line in lines:
        s = line.strip()
        # dropped lines become blank lines so that #line keeps the numbering
        if s == "module;":
            out.append("")
            continue
        if re.match(r"^(export\s+)?module\s+[\w.]+\s*;", s):
            out.append("")
            continue
        if re.match(r"^(export\s+)?import\s+[\w.:<>\"]+\s*;", s):
            out.append("")
            continue
        m = re.match(r'^#include\s+"([^"]+)"', s)
        if m and os.path.basename(m.group(1)) in DROP_INCLUDES:
            out.append("")
            continue
        out.append(line)
    out = unwrap_export_blocks(out)
    res = []
    for line in out:
        line = re.sub(r"^(\s*)export\s+(?=(class|struct|enum|auto|constexpr|inline|using|template|double|int|void|namespace|const|std::))",
                      r"\1", line)
        res.append(line)
    text = "\n".join(res) + "\n"

    if path.endswith("pseudo/io/upf.cppm"):
        # keep the data structs and the class definition, drop the pugixml parser
        cut = text.find("\nnamespace {")
        if cut < 0:
            raise SystemExit("refgen: could not find UPF parser body")
        text = text[:cut] + "\n// [refgen] pugixml-based UPF parser body removed; UPF::UPF is defined by oracle/ref_driver.cpp\n"
    if path.endswith("pseudo/ncpp_advance.cppm"):
        text = text.replace("\nprivate:\n", "\npublic:  // [refgen] opened for table export\n")
    return text


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EFFMASS_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        raise SystemExit("refgen: give the reference checkout's root (argument or EFFMASS_REFERENCE)")
    os.makedirs(OUT_DIR, exist_ok=True)
    parts = ['// Generated by oracle/refgen.py from the reference sources. Do not commit.\n',
             '#include "../ref_shims.hpp"\n']
    with open(os.path.join(ref, "src/physical_constants.hpp"), encoding="utf-8") as f:
        parts.append('#line 1 "src/physical_constants.hpp"\n' + f.read().replace("#pragma once", "") + "\n")
    for rel in ORDER:
        p = os.path.join(ref, rel)
        with open(p, encoding="utf-8") as f:
            src = f.read()
        parts.append(f"\n// ===== [refgen] {rel} =====\n")
        parts.append(f'#line 1 "{rel}"\n')
        parts.append(transform(rel, src))
    dst = os.path.join(OUT_DIR, "ref_all.cpp")
    with open(dst, "w", encoding="utf-8") as f:
        f.write("".join(parts))
    print(dst)


if __name__ == "__main__":
    main()

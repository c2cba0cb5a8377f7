"""Build recipe for ``oracle/_ref``: the reference's own code, made runnable here.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``geepee_gb300``) imports,
links or runs anything under ``oracle/``.

The reference (thangbui/geepee) is Python 2 code whose only native part is a
``scipy.weave`` C++ loop; neither Python 2 nor weave exists in this image.  This
script reads the reference sources from ``--src`` (default: ``$GEEPEE_REFERENCE``)
and writes two artefacts into ``oracle/_ref/`` (git-ignored, never committed):

1. ``oracle/_ref/geepee_ref/`` - a Python 3 / numpy 2 package made from
   ``geepee/{config,utils,kernels,lik_layers,base_models,aep_models,vfe_models}.py``
   by mechanical edits only:

   * ``print x``  ->  ``print(x)``; ``cPickle`` -> ``pickle``; ``__builtin__`` -> ``builtins``;
   * ``M * (M + 1) / 2``  ->  ``M * (M + 1) // 2`` (array sizes must be integers);
   * implicit relative imports -> explicit package-relative imports;
   * ``import weave`` / ``import matplotlib.pyplot`` removed (both are absent here);
   * ``float(sf)`` on a shape-(1,) array -> ``float(np.ravel(sf)[0])`` (numpy 2 refuses it);
   * ``np.linalg.solve(S[D,M,M], m[D,M])`` -> solve against ``m[..., None]`` and take
     ``[..., 0]`` (numpy 2 treats a 2-D right-hand side as a matrix);
   * the weave-backed ``compute_psi_weave`` is rebound to the reference's own numpy
     ``psi1computations`` / ``psi2computations`` (``geepee/kernels.py:317-352``), which
     compute the same statistics.

2. ``oracle/_ref/psi_weave_ref.cpp`` - the C++ body of ``compute_psi_weave``
   (``geepee/kernels.py:201-234``) extracted verbatim from the reference source and
   wrapped in a C function with blitz-style ``a(i, j)`` accessors, so that the
   reference's own native loop can be compiled with g++ and timed/checked.

Usage:  python oracle/make_ref.py --src /path/to/reference   (or set GEEPEE_REFERENCE)
"""
from __future__ import annotations

import argparse
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MODULES = ["config", "utils", "kernels", "lik_layers", "base_models",
           "aep_models", "vfe_models"]


def _py3(text: str, name: str) -> str:
    out = []
    for line in text.splitlines():
        m = re.match(r"^(\s*)print (?!\()(.*)$", line)
        if m:
            line = f"{m.group(1)}print({m.group(2)})"
        out.append(line)
    text = "\n".join(out) + "\n"
    text = text.replace("import cPickle as pickle", "import pickle")
    text = text.replace("import __builtin__", "import builtins as __builtin__")
    text = text.replace("M * (M + 1) / 2", "M * (M + 1) // 2")
    text = text.replace("self.M * (self.M + 1) / 2", "self.M * (self.M + 1) // 2")
    text = re.sub(r"^import weave\s*$", "weave = None", text, flags=re.M)
    text = re.sub(r"^import matplotlib\.pyplot as plt\s*$", "plt = None", text, flags=re.M)
    for mod in MODULES:
        text = re.sub(rf"^(\s*)from {mod} import", rf"\1from .{mod} import", text, flags=re.M)
    text = re.sub(r"float\((sf2?)\)", r"float(np.ravel(\1)[0])", text)
    if name == "aep_models":
        # numpy-2 solve semantics: (D,M,M) \ (D,M) must be a batch of vectors
        text = text.replace("np.linalg.solve(\n            self.Su, self.mu))",
                            "np.linalg.solve(\n            self.Su, self.mu[..., None])[..., 0])")
        text = text.replace("np.linalg.solve(\n            self.Suhat, self.muhat))",
                            "np.linalg.solve(\n            self.Suhat, self.muhat[..., None])[..., 0])")
    if name == "lik_layers":
        text = text.replace("VinvY = np.linalg.solve(Vy, Ydiff)",
                            "VinvY = np.linalg.solve(Vy, Ydiff[..., None])[..., 0]")
    if name == "kernels":
        text += (
            "\n\n# --- shim: weave is unavailable; bind the reference's own numpy psi\n"
            "# statistics (kernels.py:317-352), which compute the same quantities.\n"
            "def compute_psi_weave(lls2, lsf2, xmean, xvar, z):\n"
            "    sf2 = float(np.exp(np.ravel(lsf2)[0]))\n"
            "    ell = np.exp(0.5 * np.asarray(lls2))\n"
            "    return (psi1computations(sf2, ell, z, xmean, xvar),\n"
            "            psi2computations(sf2, ell, z, xmean, xvar))\n"
        )
    return text


_CPP_PRELUDE = r"""// GENERATED by oracle/make_ref.py from the reference's geepee/kernels.py
// (compute_psi_weave C++ body, kernels.py:201-234).  Not committed.
#include <math.h>
struct A1 { const double* p; double operator()(int i) const { return p[i]; } };
struct A2 { double* p; int s; double& operator()(int i, int j) const { return p[(long)i * s + j]; } };
struct A3 { double* p; int s0, s1;
            double& operator()(int i, int j, int k) const { return p[(long)i * s0 + (long)j * s1 + k]; } };
extern "C" void ref_psi_weave(double* psi1_p, double* psi2_p, int M, int Q, int N, double sf2,
                              const double* ls2_p, const double* z_p, const double* xmean_p,
                              const double* xvar_p, const double* ld1_p, const double* ld2_p) {
  A2 psi1{psi1_p, M};
  A3 psi2{psi2_p, M * M, M};
  A1 ls2{ls2_p};
  A2 z{(double*)z_p, Q}, xmean{(double*)xmean_p, Q}, xvar{(double*)xvar_p, Q};
  A2 log_denom_psi1{(double*)ld1_p, Q}, log_denom_psi2{(double*)ld2_p, Q};
"""


def _extract_weave_body(kernels_src: str) -> str:
    start = kernels_src.index("def compute_psi_weave(")
    seg = kernels_src[start:]
    m = re.search(r'\n\s*code = """(.*?)"""', seg, flags=re.S)
    if m is None:
        raise RuntimeError("could not find the weave code block of compute_psi_weave")
    return m.group(1)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=os.environ.get("GEEPEE_REFERENCE"), required=not os.environ.get("GEEPEE_REFERENCE"),
                    help="the reference checkout (default: $GEEPEE_REFERENCE)")
    args = ap.parse_args(argv)
    src = os.path.join(args.src, "geepee")
    if not os.path.isdir(src):
        print(f"make_ref: reference not found at {src}; nothing built", file=sys.stderr)
        return 1
    pkg = os.path.join(OUT, "geepee_ref")
    os.makedirs(pkg, exist_ok=True)
    for mod in MODULES:
        with open(os.path.join(src, mod + ".py")) as f:
            text = f.read()
        with open(os.path.join(pkg, mod + ".py"), "w") as f:
            f.write(_py3(text, mod))
        if mod == "kernels":
            body = _extract_weave_body(text)
            with open(os.path.join(OUT, "psi_weave_ref.cpp"), "w") as f:
                f.write(_CPP_PRELUDE + body + "\n}\n")
    with open(os.path.join(pkg, "__init__.py"), "w") as f:
        f.write("# generated by oracle/make_ref.py (reference code, Python 3 shim)\n")
    print(f"make_ref: wrote {pkg} and psi_weave_ref.cpp")
    return 0


if __name__ == "__main__":
    sys.exit(main())

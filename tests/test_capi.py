"""The C ABI library loads and exports every symbol its headers declare (no GPU needed)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(nlm_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(nlm):
    lib = ctypes.CDLL(os.path.join(ROOT, "multimodenonlinearoptics_gb300", "libnlm_gb300.so"))
    syms = declared_symbols()
    assert len(syms) > 20
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_solver_registry_matches_reference_order(nlm):
    # solvers/RegisteredSolvers.hpp:1-16
    assert nlm.SOLVERS == ["Chi3", "Chi2PDC", "Chi2SFG", "Chi2AFC", "Chi2SFGPDC", "Chi2SFGII", "Chi2PDCII",
                           "Chi2SFGOPA", "Chi2SFGXPM", "Chi2SHG", "Chi2SHGOPA", "Chi2DSFG", "Chi2SHGXPM", "Chi2ASHG",
                           "Chi3GNLSE"]

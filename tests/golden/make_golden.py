"""Generate golden vectors from the reference's own NumPy prototype.

Reads prototype/xpbi2d.py of Chiplis/xpbi-webgpu (checkout given as
argv[1], else XPBI_REFERENCE, else `reference` beside this repository),
extracts its `drucker_prager` (xpbi2d.py:93-108)
and `stvk_psi_and_dpsi` (xpbi2d.py:110-116) with `ast` — the script's
simulation loop is not executed — and evaluates them with the dimension
set to 3 (the functions are written for any `d`) on seeded singular-value
triples. The result is committed as dp_stvk_prototype.json and pins the
oracle's Drucker-Prager return map and StVK-Hencky energy.

Inputs keep every singular value in [0.55, 1.8] so the reference's two
clamps (WGSL safeSig [1e-3, 1e3], prototype max(S, 1e-10)) never act, and
never hit a zero deviator, where the WGSL projects to the tip and the
prototype does not (common.js:213 vs xpbi2d.py:101-107).
"""
from __future__ import annotations

import ast
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_functions(ref_root: str):
    path = os.path.join(ref_root, "prototype", "xpbi2d.py")
    tree = ast.parse(open(path).read(), filename=path)
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef)
            and n.name in ("drucker_prager", "stvk_psi_and_dpsi")]
    assert len(keep) == 2, "prototype functions not found"
    return ast.Module(body=keep, type_ignores=[])


def main():
    repo = os.path.dirname(os.path.dirname(HERE))
    ref_root = (sys.argv[1] if len(sys.argv) > 1 else
                os.environ.get("XPBI_REFERENCE") or os.path.join(os.path.dirname(repo), "reference"))
    mod = load_functions(ref_root)
    rng = np.random.default_rng(2024)
    cases = []
    for E, nu, phi in [(2000.0, 0.3, 35.0), (1e5, 0.3, 30.0), (2e5, 0.3, 35.0), (5e4, 0.25, 25.0)]:
        mu = E / (2 * (1 + nu))
        lam = E * nu / ((1 + nu) * (1 - 2 * nu))
        alpha = math.sqrt(2.0 / 3.0) * 2.0 * math.sin(math.radians(phi)) / (3.0 - math.sin(math.radians(phi)))
        ns = {"np": np, "d": 3, "mu": mu, "lam": lam, "alpha_dp": alpha}
        exec(compile(mod, "xpbi2d.py", "exec"), ns)
        S = rng.uniform(0.55, 1.8, size=(256, 3))
        # bias a quarter of the cases into compression (tr(log S) < 0) so all
        # three return-map cases occur
        S[:64] = rng.uniform(0.55, 1.05, size=(64, 3))
        S = -np.sort(-S, axis=1)
        dp = ns["drucker_prager"](S.copy())
        psi, dpsi = ns["stvk_psi_and_dpsi"](S.copy())
        cases.append(dict(E=E, nu=nu, phi=phi, mu=mu, lam=lam, alpha=alpha, sigma=S.tolist(), dp=dp.tolist(),
                          psi=psi.tolist(), dpsi=dpsi.tolist()))
    out = dict(source="prototype/xpbi2d.py:93-116 evaluated with d=3", cases=cases)
    with open(os.path.join(HERE, "dp_stvk_prototype.json"), "w") as f:
        json.dump(out, f)
    print("wrote", sum(len(c["sigma"]) for c in cases), "vectors")


if __name__ == "__main__":
    main()

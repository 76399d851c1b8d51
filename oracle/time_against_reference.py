"""Times the oracle's Crystal path against the reference's own on the same problems (CPU only).

Run where the reference source is available (read-only), from the repository root:

    python oracle/time_against_reference.py /path/to/reference [count]

Both solve ``count`` seeded in-cone problems of the 11x11 batched sweep (the bench's CPU
sample: ``numpy.random.default_rng(1)``), each as set_source + solve + poynting_flux_end for
te and again for tm, after one untimed solve.  Prints solves/s of each and the largest
difference of their R and T.  This is how the bench's reference arm, which runs the oracle
because the reference cannot travel to the GPU machine, is checked to be no slower than the
reference itself.  The reference imports numba at module load; ``tests/golden/_shim`` provides
an identity ``njit`` (the decorated functions are not on the Crystal solve path).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main(ref_root, count=6):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "_shim"))
    sys.path.insert(0, ref_root)
    from khepri.crystal import Crystal  # the reference
    from khepri_gb300 import workloads
    from oracle import khepri_oracle as ko

    st = workloads.batched_structure(0)
    wl, kp = workloads.batched_problems()
    inside = np.flatnonzero(np.hypot(kp[:, 0], kp[:, 1]) < 2 * np.pi / wl)
    probs = np.random.default_rng(1).choice(inside, count, replace=False)

    def build(cls):
        cl = cls(st.pw)
        for name, (kind, eps, depth) in st.layers.items():
            (cl.add_layer_uniform if kind == "uniform" else cl.add_layer_pixmap)(name, eps, depth)
        cl.set_device(st.stack, False)
        return cl

    results = {}
    for name, cl in (("reference", build(Crystal)), ("oracle", build(ko.OracleCrystal))):
        cl.set_source(wl[probs[0]], 1.0, 0.0, kp=tuple(kp[probs[0]]))
        cl.solve()
        cl.poynting_flux_end()
        out = []
        t0 = time.perf_counter()
        for p in probs:
            cl.set_source(wl[p], 1.0, 0.0, kp=tuple(kp[p]))
            cl.solve()
            r_te, t_te = cl.poynting_flux_end()
            cl.set_source(wl[p], 0.0, 1.0, kp=tuple(kp[p]))  # same S-matrix, tm source
            r_tm, t_tm = cl.poynting_flux_end()
            out.append((float(r_te), float(t_te), float(r_tm), float(t_tm)))
        dt = time.perf_counter() - t0
        results[name] = np.array(out)
        print(f"{name}: {count / dt:.3f} solves/s ({dt:.2f} s for {count} problems, both polarisations)")
    print("max |dR|, |dT| (both polarisations):", float(np.abs(results["reference"] - results["oracle"]).max()))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python oracle/time_against_reference.py /path/to/reference [count]")
    main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 6)

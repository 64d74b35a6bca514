"""FP64 reference energies at sizes the CPU reference cannot hold (run on a GPU).

The reference keeps the full nmo^4 ERI and L in host memory (about 214 GB at no=40,
nv=300), so its converged energies at the large sizes come from this engine's FP64 path
instead: the DMMA FP64 kernels, which reproduce the reference to 1e-12 (residuals) and
1e-10 Eh (energies) where both run (tests/test_gpu_ccsd.py).  Output:
``tests/golden/fp64_reference.json`` keyed "no_nv_seed".

Usage: python tests/golden/make_fp64_reference.py [--triples] [no nv seed] ...

With ``--triples`` the FP64 (T) energy (multi-term DMMA path) is added for each size.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(argv):
    import torch
    import pycc_gb300 as pg
    triples = "--triples" in argv
    argv = [a for a in argv if a != "--triples"]
    sizes = [(40, 300, 2)]
    if len(argv) >= 3:
        vals = [int(x) for x in argv]
        sizes = [tuple(vals[i:i + 3]) for i in range(0, len(vals), 3)]
    out_path = os.path.join(HERE, "fp64_reference.json")
    refs = json.load(open(out_path)) if os.path.exists(out_path) else {}
    for no, nv, seed in sizes:
        fac = pg.SyntheticFactors(no, nv, seed, coupling="matched")
        H = pg.Hamiltonian.from_factors(fac, device="cuda:0")
        w = pg.CCwfn(H, precision="DP")
        t0 = time.time()

        def cb(n, e, de, rms):
            print("fp64 %d %d: it %d E %.12f dE %.2e rms %.2e (%.0f s)"
                  % (no, nv, n, e, de, rms, time.time() - t0), flush=True)
        e = w.solve_cc(1e-9, 1e-7, 60, callback=cb)
        rec = {"ecc": e, "niter": w.niter, "e_conv": 1e-9, "r_conv": 1e-7,
               "coupling": fac.coupling, "s_per_iter": sum(w.iter_times) / len(w.iter_times),
               "energies": w.energies}
        if triples:
            from pycc_gb300.triples import t_energy_fp64
            t0 = time.time()
            rec["et"] = t_energy_fp64(w)
            torch.cuda.synchronize()
            rec["t_s"] = time.time() - t0
            print("fp64 (T) %d %d: %.12f (%.0f s)" % (no, nv, rec["et"], rec["t_s"]), flush=True)
        refs["%d_%d_%d" % (no, nv, seed)] = rec
        with open(out_path, "w") as f:
            json.dump(refs, f, indent=1)
        del w, H
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main(sys.argv[1:])

"""Generate tests/golden/ref_fixtures.npz from the reference's own code.

Builds oracle/_ref/smaiso_wcomp_ref (oracle/build_ref.sh: smaiso-wcomp.cpp compiled
against the MPI/FFTW-MPI stand-in in oracle/refshim/, with the run-size
substitutions listed there), runs every case of tests/golden/ref_cases.py as the
stated number of MPI ranks, and stores the sampled fields, their norms and the
full-precision diagnostics. Needs the reference source (default
/root/reference/smaiso-wcomp.cpp, or SWC_REFERENCE_SRC).

Run: python tests/golden/make_ref_fixtures.py [--all]
(without --all, the cases already in the file are kept and only new ones are run)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import ref_run  # noqa: E402
from smaiso_wcomp_gb300.abi import default_params, derived  # noqa: E402
import ref_cases  # noqa: E402


def main():
    path = os.path.join(HERE, "ref_fixtures.npz")
    out = {}
    if "--all" not in sys.argv and os.path.exists(path):
        out = dict(np.load(path))
    for case, c in ref_cases.CASES.items():
        if f"{case}.diag" in out:
            continue
        p = default_params(*c["shape"])
        d = derived(p)
        if c["ic"] == "ref":   # the reference's own initial state: no psi file
            prof, psi0 = {}, None
        else:
            prof = ref_cases.profiles(case, d["dx"], d["dz"])
            psi0 = ref_cases.initial_psi(prof, c["shape"], c["seed"], c["noise"])
        res = ref_run.run(c["shape"], c["ranks"], c["steps"], sorted(c["dumps"]), psi0=psi0)
        for k, v in prof.items():
            out[f"{case}.{k}"] = v
        out[f"{case}.diag"] = np.array(res["diag"], dtype=np.float64)
        for step, size in c["dumps"].items():
            idx = ref_cases.sample_index(case, step, size)
            for f in ref_cases.fields_at(step):
                full = res["fields"][step][f]
                out[f"{case}.s{step}.{f}"] = full.reshape(-1)[idx]
                out[f"{case}.s{step}.{f}.norm"] = np.float64(np.linalg.norm(full))
        print(f"{case}: {c['shape']} x {c['ranks']} ranks, {c['steps']} steps, "
              f"diag rows {len(res['diag'])}", flush=True)
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


if __name__ == "__main__":
    main()

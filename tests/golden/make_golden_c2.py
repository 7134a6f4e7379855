"""Generate the FP64 oracle fixture of the 1005 x 1005 x 51 workload (Nnum 15, 67 x 67
lenslets, 51 planes 0..200 um, plane k PSF window 31+4k, K0 231, 2000 somas, seed 0).

    python tests/golden/make_golden_c2.py [max_iter]

The full volume (51.5 M voxels, 412 MB in FP64) is too large to commit, so the fixture
holds the measured image (Poisson counts), a fixed random sample of 131072 voxel indices
with their oracle values after 3 (and, when max_iter >= 10, 10) iterations, and per-plane
sums and the L2 norm of each oracle volume.  The PSF is regenerated from the seed by the
tests (mesolf_gb300.synth.config2).  The RL view step runs in the C/OpenMP port of the
oracle (oracle/mlf_oracle.c, checked against the numpy restatement in tests/test_oracle.py);
the rest of the solve (normalisation, realignment, weights, spiral, sample_filter) is the
numpy oracle.  One iteration takes ~15 min on 8 x86 cores.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import cbuild  # noqa: E402
from oracle import mesolf_ref as R  # noqa: E402
from mesolf_gb300 import synth  # noqa: E402

NAME = "lf1005x1005x51_k231.npz"
NSAMPLE = 131072


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main(max_iter=3):
    t0 = time.time()
    cbuild.build()
    w = synth.config2()
    H, Ht = w.psf()
    LF = w.measured(H, w.volume())
    assert LF.max() < 65535 and np.array_equal(LF, np.round(LF))
    print(f"inputs ready {time.time() - t0:.0f} s", flush=True)
    n = LF.shape[0] * LF.shape[1] * w.Z
    idx = np.sort(np.random.default_rng(7).choice(n, NSAMPLE, replace=False)).astype(np.uint32)
    payload = dict(lf=LF.astype(np.uint16), idx=idx)
    path = os.path.join(HERE, NAME)

    def save(it, X):
        flat = X.reshape(-1, order="F")
        payload[f"x{it}"] = flat[idx].astype(np.float32)
        payload[f"plane_sums{it}"] = X.sum(axis=(0, 1))
        payload[f"l2_{it}"] = np.float64(np.linalg.norm(flat))
        np.savez_compressed(path, **payload)
        man = os.path.join(HERE, "manifest.json")
        m = json.load(open(man))
        m[NAME] = sha(path)
        json.dump(m, open(man, "w"), indent=1)
        print(f"iteration {it} saved {time.time() - t0:.0f} s", flush=True)

    def cb(it, X):
        print(f"iteration {it + 1} done {time.time() - t0:.0f} s", flush=True)
        if it + 1 in (3, 10):
            save(it + 1, X)

    R.recon_phase_space(LF, H, Ht, max_iter, callback=cb, view_step=cbuild.view_step)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 3)

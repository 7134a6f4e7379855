"""Generate the committed golden fixtures from the FP64 oracle (run on a CPU host).

    python tests/golden/make_golden.py

Fixtures (npz, float32 payloads; SHA-256 of each file in manifest.json):
  lf165x165x21_k61.npz   config "Nnum 15, 11x11 lenslets, 21 planes, K0 61": measured image,
                         oracle volume after 2 and 8 RL iterations, view weights
  small_views.npz        per-view forward / backward projections on a 5 x 4 lenslet,
                         3-plane, K0 61 case for views (7,7), (0,0), (14,3)
The PSF and volume are regenerated from the seed (mesolf_gb300.synth) by the tests.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import mesolf_ref as R  # noqa: E402
from mesolf_gb300 import synth  # noqa: E402


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    out = {}
    w = synth.config1()
    H, Ht = w.psf()
    LF = w.measured(H, w.volume())
    snaps = {}
    R.recon_phase_space(LF, H, Ht, 8, callback=lambda it, X: snaps.__setitem__(it + 1, X.copy()))
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, Htc = R.gen_phasespace_psf(Hn, Htn)
    p = os.path.join(HERE, "lf165x165x21_k61.npz")
    np.savez_compressed(p, lf=LF.astype(np.float32), x2=snaps[2].astype(np.float32),
                        x8=snaps[8].astype(np.float32), weights=R.view_weights(Hps),
                        psf_sum=np.float64(H.astype(np.float64).sum()))
    out[os.path.basename(p)] = sha(p)

    ws = synth.small_config(lenslets=(5, 4), K0=61, Z=3)
    H, Ht = ws.psf()
    Hn, Htn = R.normalize_psf(H, Ht)
    Hps, Htc = R.gen_phasespace_psf(Hn, Htn)
    rng = np.random.default_rng(42)
    vol = rng.random((75, 60, 3))
    proj = rng.random((5, 4))
    views = [(7, 7), (0, 0), (14, 3)]
    fw = np.stack([R.forward_ps(Hps[:, :, u, v, :], vol, 15) for u, v in views])
    bw = np.stack([R.backward_ps(Htc[:, :, u, v, :], proj, u, v, 15) for u, v in views])
    p = os.path.join(HERE, "small_views.npz")
    np.savez_compressed(p, vol=vol.astype(np.float32), proj=proj.astype(np.float32),
                        views=np.array(views), fwd=fw.astype(np.float32), bwd=bw.astype(np.float32),
                        vol64=vol, proj64=proj)
    out[os.path.basename(p)] = sha(p)
    json.dump(out, open(os.path.join(HERE, "manifest.json"), "w"), indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()

"""Extract the reference's own MEX test input, ``src/cuda/vols_slice.mat`` (one
``mex_lfm_convolution_vec`` bitmap argument from a seed-library run: 376 x 376 x 77 single,
saved as a gpuArray), into ``tests/golden/vols_slice_sparse.npz`` (column-major flat indices
of the non-zeros and their values), so that the parity tests can run the reference kernel
and this library's projector on it where the reference tree is absent.

    python tests/golden/make_ref_fixture.py

The gpuArray is stored as a MATLAB opaque object whose data sits in the file's subsystem
stream as one miSINGLE element of 376*376*77 floats; this finds that element by its tag.
"""
import hashlib
import json
import os
import struct

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.environ.get("MLF_REFERENCE_ROOT", "/root/reference"), "src", "cuda", "vols_slice.mat")
OUT = os.path.join(HERE, "vols_slice_sparse.npz")
SHAPE = (376, 376, 77)


def extract(path=SRC):
    stream = sio.loadmat(path)["__function_workspace__"].tobytes()
    nbytes = 4 * int(np.prod(SHAPE))
    at = stream.find(struct.pack("<II", 7, nbytes))  # miSINGLE tag
    if at < 0:
        raise ValueError("no single-precision element of the expected size in the subsystem stream")
    return np.frombuffer(stream[at + 8:at + 8 + nbytes], dtype="<f4").reshape(SHAPE, order="F")


def main():
    a = extract()
    flat = a.reshape(-1, order="F")
    idx = np.flatnonzero(flat).astype(np.int32)
    np.savez_compressed(OUT, shape=np.array(SHAPE, np.int64), index=idx, value=flat[idx].astype(np.float32))
    man_path = os.path.join(HERE, "manifest.json")
    man = json.load(open(man_path))
    man[os.path.basename(OUT)] = hashlib.sha256(open(OUT, "rb").read()).hexdigest()
    json.dump(man, open(man_path, "w"), indent=1)
    print(OUT, "nnz", idx.size, "sum", float(flat.sum(dtype=np.float64)), "max", float(flat.max()))


if __name__ == "__main__":
    main()

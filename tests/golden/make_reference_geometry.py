"""Copy the reference's own serpentine geometry into a compressed test fixture.

    python tests/golden/make_reference_geometry.py [REFERENCE_ROOT]

The reference ships the geometry of its microfluidics example as two raw files that finit
reads with read_var (microfluidics_complex_domain/finit.f90:98-128, inout.f90:75-86):

* domain_snake_420_180.bin       the solid mask in {-1, 1} (1 in the walls)
* domain_snake_420_180_dist.bin  the distance to the walls, bdr_ph_dist

Each is 420 x 180 little-endian float64 values written as ((var(i,k),k=1,nz),i=1,nr), that is
a C-order [nr][nz] array.  They are the only reference-held inputs of the solver path.  The
GPU machine has no copy of the reference, so the values are stored here unchanged (bit for bit,
zlib-compressed: 22 KB instead of 1.2 MB) as domain_snake_420_180.npz with arrays `mask` and
`dist`, both of shape (nr, nz) = (420, 180).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NR, NZ = 420, 180
FILES = {"mask": "domain_snake_420_180.bin", "dist": "domain_snake_420_180_dist.bin"}


def read_var(path, nr=NR, nz=NZ):
    """read_var (inout.f90:75-86): stream of ((var(i,k),k=1,nz),i=1,nr) -> array [i][k]."""
    a = np.fromfile(path, dtype="<f8")
    if a.size != nr * nz:
        raise ValueError(f"{path}: {a.size} values, expected {nr * nz}")
    return a.reshape(nr, nz)


def main(ref_root="/root/reference"):
    src = os.path.join(ref_root, "microfluidics_complex_domain")
    arrays = {k: read_var(os.path.join(src, f)) for k, f in FILES.items()}
    out = os.path.join(HERE, "domain_snake_420_180.npz")
    np.savez_compressed(out, **arrays)
    print(out, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main(*sys.argv[1:])

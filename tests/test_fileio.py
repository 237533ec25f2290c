"""The driver's files (CPU only: the host code of the C library, no GPU call).

* The `input` deck: list-directed READ of the first value per line (mcl6.f90:68-100), with the
  deck's trailing '!' notes, quoted characters and Fortran exponents.
* Checkpoints: `output` writes Fortran unformatted sequential records (4-byte length markers)
  ((a(i,k),k=0,N),i=0,M) of x, y, u, v, p, f, f2 and t (inout.f90:1-19).  They are read back
  here by an independent numpy reader that follows the reference's own post-processing reader
  (microfluidics_complex_domain/post_process/da1.py:7-37: skip the marker, read (nr+1)(nz+1)
  doubles, skip two markers, ...).  `input` takes t from the record after f (inout.f90:56), which
  is f2's first value.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi, fileio
from drd_application_gb300.layout import cell_shape, u_shape, v_shape

DECK = """5.0E-2 !5.0E-4 ! 0.05 !xld
1 !00 !32 !re
100 !.0  !10 !ca
50000.    !vs
0.0 !0.038 !xls
0.0 !0.038 !xls
0  !0.0038 !xls
0  !0.0038 !xls
0.0  !0.2 ! uw top
0.0  !-0.2 ! uw bottom
3.5  !1.0 !slen
1.5  !1.0 !shig

135 !45 ! contact angle
1.0 !0.38 ! slipratio
0  !iflag
10 !0 !step to output
30000 !tf
0.005 !0.01 !interface thickness
1.5 !1.0 ! stability
1.0D-8  !! tolerance
0 !-10. !external force z
0. !-10. !external force x
0.1 !1.0 !time step change
1. !000. !density ratio
100 !300 !viscosity ratio
1.0 !0.2   ! UU
'n' ! lr_bd_type
'd' ! top_type_ph
'd' ! bot_type_ph
'n'   ! top_type_u
'n'   ! bot_type_u
"""


@pytest.fixture(scope="module")
def lib(cuda_lib):
    return cuda_lib


def test_deck_parses_first_values(lib, tmp_path):
    f = tmp_path / "input"
    f.write_text(DECK)
    d = fileio.read_deck(f)
    assert d.entries == 31
    assert (d.xld, d.re, d.ca, d.vs, d.slen, d.shig, d.angle) == (0.05, 1.0, 100.0, 50000.0, 3.5, 1.5, 135.0)
    assert (d.iflag, d.istep, d.tf, d.I_thickness, d.tol) == (0, 10, 30000.0, 0.005, 1.0e-8)
    assert (d.ggz, d.ggx, d.time_step_change, d.lambda_rho, d.lambda_eta, d.UU) == (0.0, 0.0, 0.1, 1.0, 100.0, 1.0)
    assert (d.lr_bd_type, d.top_type_ph, d.bot_type_ph, d.top_type_u, d.bot_type_u) == (b"n", b"d", b"d", b"n", b"n")
    # the TP deck's extra line (two_phase_flow_complex_domain/mcl6.f90:100)
    f.write_text(DECK + "'y'   ! complex domain\n")
    assert fileio.read_deck(f).is_complex_domain == b"y" and fileio.read_deck(f).entries == 32


def test_deck_to_params(lib, tmp_path):
    f = tmp_path / "input"
    f.write_text(DECK)
    p = fileio.params_from_deck(fileio.read_deck(f), 420, 180)
    assert p.dr == 3.5 / 420 and p.dz == 1.5 / 180
    assert p.dt == min(3.5 / 420, 1.5 / 180) * 0.1  # finit.f90:395-397
    assert (p.twall, p.penalty_k, p.lr_bd_type) == (0.1, 1.0e5, ord("n"))


def test_deck_errors(lib, tmp_path):
    f = tmp_path / "input"
    f.write_text(DECK.replace("30000 !tf", "abc !tf"))
    with pytest.raises(ValueError, match="tf"):
        fileio.read_deck(f)
    f.write_text("\n".join(DECK.splitlines()[:10]))
    with pytest.raises(ValueError, match="31"):
        fileio.read_deck(f)
    with pytest.raises(ValueError):
        fileio.read_deck(tmp_path / "missing")


def _da1_reader(path, nr, nz):
    """Independent reader of an `output` file: 4-byte markers around each record."""
    raw = open(path, "rb").read()
    recs, pos = [], 0
    while pos < len(raw):
        n = int.from_bytes(raw[pos:pos + 4], "little")
        recs.append(np.frombuffer(raw[pos + 4:pos + 4 + n], dtype="<f8"))
        assert int.from_bytes(raw[pos + 4 + n:pos + 8 + n], "little") == n
        pos += n + 8
    fields = [r.reshape(nr + 1, nz + 1) for r in recs[:7]]  # [i][k]: k fastest
    return fields, recs[7]


def test_output_records_and_input_quirk(lib, tmp_path):
    nr, nz, dr, dz = 12, 7, 0.25, 0.5
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal(u_shape(nr, nz)), rng.standard_normal(v_shape(nr, nz))
    p, f, f2 = (rng.standard_normal(cell_shape(nr, nz)) for _ in range(3))
    path = tmp_path / "data001"
    fileio.output(path, nr, nz, dr, dz, u, v, p, f, f2, 1.25)
    fields, trec = _da1_reader(path, nr, nz)
    assert trec.tolist() == [1.25]
    ii, kk = np.meshgrid(np.arange(nr + 1), np.arange(nz + 1), indexing="ij")
    assert np.array_equal(fields[0], (ii + 0.5) * dr) and np.array_equal(fields[1], (kk + 0.5) * dz)
    # u(i,k) at [k+1, i+1] of UFACE, v(i,k) at [k, i+1] of VFACE, CELL at [k+1, i+1]
    assert np.array_equal(fields[2], u[1:nz + 2, 1:nr + 2].T)
    assert np.array_equal(fields[3], v[0:nz + 1, 1:nr + 2].T)
    for got, a in zip(fields[4:], (p, f, f2)):
        assert np.array_equal(got, a[1:nz + 2, 1:nr + 2].T)
    back = fileio.input(path, nr, nz)
    assert np.array_equal(back["u"][1:nz + 2, 1:nr + 2], u[1:nz + 2, 1:nr + 2])
    assert np.array_equal(back["f"][1:nz + 2, 1:nr + 2], f[1:nz + 2, 1:nr + 2])
    assert back["t"] == f2[1, 1]  # f2(0,0): the reference's restart quirk (inout.f90:56)
    assert fileio.read_time(path, nr, nz) == 1.25


def test_output_particles_record(lib, tmp_path):
    pp = abi.default_particle_params(3.5, 1.5)
    pts = np.array(abi.particle_chain(pp, 1.75, 0.42))
    path = tmp_path / "part001"
    fileio.output_particles(path, pts)
    raw = open(path, "rb").read()
    assert int.from_bytes(raw[:4], "little") == 18 * 8 and int.from_bytes(raw[-4:], "little") == 18 * 8
    # ((points(i,k),i=0,Np-1),k=0,1): all x, then all y
    assert np.array_equal(np.frombuffer(raw[4:-4], dtype="<f8"), pts.reshape(-1))

"""AllCells plot output (3_6/ModSavePlot.f90:520-650) and the binary restart.

CPU: the oracle's restatement of ModSave_AllCells is pinned against a numpy
restatement of the same formulas (corner averages of 8 cells, face
coordinates of 3_6/ModBlock.f90:320-322, Cartesian position and vectors with
the Yang mapping) and against the Fortran ES16.8 text layout, including the
three-digit-exponent form. GPU: the library's files equal the oracle's byte
for byte in FP64, agree numerically in mixed precision, and a restart dump
continues the run bit for bit.
"""
import os
import re

import numpy as np
import pytest

import falcon_gb300 as fg
import oracle
from falcon_gb300 import config, synth

RSUN = float(np.float32(6.955e10))
FIELD = re.compile(r"^ *-?\d\.\d{8}(E[+-]\d\d|[+-]\d\d\d)$")


def parse_block(path):
    """Lines of 12 ES16.8 fields -> (n, 12) array; checks the field layout."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            assert len(line) == 12 * 16, len(line)
            vals = []
            for q in range(12):
                s = line[16 * q:16 * (q + 1)]
                assert FIELD.match(s), repr(s)
                t = s.strip()
                if "E" not in t:   # d.dddddddd+ddd
                    t = t[:-4] + "E" + t[-4:]
                vals.append(float(t))
            rows.append(vals)
    return np.array(rows)


def numpy_allcells(o, u, b):
    """ModSave_AllCells for block b (0-based) from the state array u."""
    t = o.cfg.tree
    ni, nj, nk = t.ni, t.nj, t.nk
    p = u[b]                                   # (9, nkp, njp, nip), Fortran i at i+1
    c = sum(p[:, dk:dk + nk + 1, dj:dj + nj + 1, di:di + ni + 1]
            for dk in (1, 2) for dj in (1, 2) for di in (1, 2)) * 0.125
    rng = o.block_ranges()[b]
    f = lambda r, n: (r[0] * (n + 1 - np.arange(1, n + 2)) + r[1] * (np.arange(1, n + 2) - 1)) / n
    r, th, ph = f(rng[0], ni), f(rng[1], nj), f(rng[2], nk)
    PH, TH, R = np.meshgrid(ph, th, r, indexing="ij")
    sth, cth, sph, cph = np.sin(TH), np.cos(TH), np.sin(PH), np.cos(PH)
    yin = bool(o.block_flags()[b] & 1)
    x0, y0, z0 = R * sth * cph, R * sth * sph, R * cth
    xyz = [x0, y0, z0] if yin else [-x0, z0, y0]
    out = [a / RSUN for a in xyz]
    for a in (1, 4):
        vx = c[a] * sth * cph + c[a + 1] * cth * cph - c[a + 2] * sph
        vy = c[a] * sth * sph + c[a + 1] * cth * sph + c[a + 2] * cph
        vz = c[a] * cth - c[a + 1] * sth
        c[a], c[a + 1], c[a + 2] = (vx, vy, vz) if yin else (-vx, vz, vy)
    cols = out + [c[v] for v in range(9)]
    return np.stack([x.reshape(-1) for x in cols], axis=1)


def _oracle_state(mk, seed=21):
    cfg = mk()
    o = oracle.Oracle(cfg)
    u = synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=seed, psi_amp=1e-3)
    o.set_state(u)
    o.exchange()
    o.exchange()
    return o


def test_oracle_allcells_matches_numpy_restatement(tmp_path):
    o = _oracle_state(config.tiny)
    d = o.save_allcells(str(tmp_path), 7)
    assert os.path.basename(d) == "AllCells_00000007"
    t = o.cfg.tree
    with open(os.path.join(d, "info.dat")) as f:
        info = f.read()
    assert info == ("nBlocks = %d\nni = %d\nnj = %d\nnk = %d\nnVarsTotal = 12\n"
                    'VARIABLES = "X [Rs]", "Y [Rs]", "Z [Rs]", "Rho1", "Vx", "Vy", "Vz", '
                    '"Bx", "By", "Bz", "S1", "PHI"\n' % (o.nblocks, t.ni, t.nj, t.nk))
    files = sorted(x for x in os.listdir(d) if x.startswith("Block_"))
    assert files[0] == "Block_00000001.dat" and len(files) == o.nblocks
    u = o.get_state()
    for b in (0, 5, o.nblocks_yin, o.nblocks - 1):   # Yin and Yang blocks
        got = parse_block(os.path.join(d, "Block_%08d.dat" % (b + 1)))
        want = numpy_allcells(o, u, b)
        assert got.shape == ((t.ni + 1) * (t.nj + 1) * (t.nk + 1), 12)
        scale = np.abs(want).max(0)
        scale[scale == 0] = 1.0
        err = (np.abs(got - want) / scale).max(0)
        assert (err <= 1e-8).all(), err


def test_oracle_allcells_three_digit_exponent(tmp_path):
    """Fortran's Ew.d drops the E before a three-digit exponent."""
    o = _oracle_state(config.tiny)
    u = o.get_state()
    u[:, 7] = 8e150       # s1 everywhere, ghosts included: every corner averages to 8e150
    u[:, 0] = -3e-120
    o.set_state(u)
    d = o.save_allcells(str(tmp_path), 1)
    with open(os.path.join(d, "Block_00000001.dat")) as f:
        line = f.readline().rstrip("\n")
    assert line[16 * 3:16 * 4] == " -3.00000000-120"
    assert line[16 * 10:16 * 11] == "  8.00000000+150"


# ---- GPU: the library's output and restart --------------------------------
def _gpu_pair(prec, divb=1, seed=23):
    mk = lambda: config.tiny(precision=prec, divb_option=divb)
    f = fg.Falcon(mk())
    o = oracle.Oracle(mk())
    u = synth.initial_state(mk(), o.block_ranges(), o.block_flags(), seed=seed, psi_amp=1e-3)
    f.upload_state(u)
    o.set_state(u)
    for x in (f, o):
        x.exchange()
        x.exchange()
    for _ in range(2):
        f.advance_rk4()
        o.step()
    return f, o


@pytest.mark.gpu
def test_gpu_allcells_fp64_byte_identical_to_oracle(tmp_path, built_lib):
    f, o = _gpu_pair(config.PREC_FP64)
    da = f.save_allcells(str(tmp_path / "gpu"), 2)
    db = o.save_allcells(str(tmp_path / "cpu"), 2)
    names = sorted(os.listdir(db))
    assert sorted(os.listdir(da)) == names and len(names) == o.nblocks + 1
    for n in names:
        with open(os.path.join(da, n), "rb") as x, open(os.path.join(db, n), "rb") as y:
            assert x.read() == y.read(), n


@pytest.mark.gpu
def test_gpu_allcells_mixed_close_to_oracle(tmp_path, built_lib):
    """Mixed precision after 2 steps: every column within 1e-5 of the oracle's,
    relative to that column's largest magnitude over the whole shell."""
    f, o = _gpu_pair(config.PREC_MIXED)
    da = f.save_allcells(str(tmp_path / "gpu"), 2)
    db = o.save_allcells(str(tmp_path / "cpu"), 2)
    n = ["Block_%08d.dat" % (b + 1) for b in range(o.nblocks)]
    x = np.concatenate([parse_block(os.path.join(da, q)) for q in n])
    y = np.concatenate([parse_block(os.path.join(db, q)) for q in n])
    s = np.abs(y).max(0)
    s[s == 0] = 1.0
    worst = (np.abs(x - y) / s).max(0)
    print("mixed AllCells vs oracle, max error / column max:", worst)
    assert (worst <= 1e-5).all(), worst


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [config.PREC_FP64, config.PREC_MIXED])
def test_gpu_restart_continues_bit_for_bit(tmp_path, built_lib, prec):
    f, _ = _gpu_pair(prec)
    path = str(tmp_path / "run.rst")
    f.save_restart(path)
    for _ in range(2):
        f.advance_rk4()
    a = f.download_state()
    g = fg.Falcon(config.tiny(precision=prec, divb_option=1))
    g.load_restart(path)
    for _ in range(2):
        g.advance_rk4()
    assert np.array_equal(a, g.download_state())


@pytest.mark.gpu
def test_gpu_restart_rejects_other_configs_and_short_files(tmp_path, built_lib):
    f, _ = _gpu_pair(config.PREC_MIXED)
    path = str(tmp_path / "run.rst")
    f.save_restart(path)
    other = fg.Falcon(config.tiny(precision=config.PREC_FP64, divb_option=1))
    before = other.download_state()
    with pytest.raises(fg.FalconError) as e:
        other.load_restart(path)
    assert e.value.code == fg.ERR_INVALID_ARG and "precision" in str(e.value)
    with open(path, "rb") as x:
        data = x.read()
    short = str(tmp_path / "short.rst")
    with open(short, "wb") as x:
        x.write(data[:-100])
    g = fg.Falcon(config.tiny(precision=config.PREC_MIXED, divb_option=1))
    with pytest.raises(fg.FalconError) as e:
        g.load_restart(short)
    assert e.value.code == fg.ERR_INVALID_ARG and "truncated" in str(e.value)
    assert np.array_equal(before, other.download_state())

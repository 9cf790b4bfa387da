"""GPU: the values cubble-cli writes — results.dat rows and snapshot columns —
recomputed independently by the FP64 oracle from the run's own state.

The reference writes, at each printed time unit (src/simulator.cu:1029-1082):
    timesPrinted  <r>/r0  N  <path>  E  dE  <vx> <vy> <vz>  |<v>|  <vr>
with E = totalEnergy() and dE = 2 |E - E_prev| / (E + E_prev), and snapshot
rows (src/simulator.cu:387-474) of
    x,y,z (minus half the box), r, vx, vy, vz, vtot, vr, path, energy,
    displacement since the previous snapshot, error, index.

cubble-cli writes its checkpoint right after a printed row (the state the
row was computed from; only the error row is reset after it), so:
  * the last results.dat row is recomputed from the checkpoint: means with
    numpy, E by the oracle on the checkpoint's pair list, dE from the E of
    the row before; agreement within 1e-12 (means of velocities, which sum
    to nearly zero, within 1e-12 of the mean magnitude), counts exact;
  * a run resumed from the checkpoint for one step writes a final snapshot;
    the oracle takes the same step from the checkpoint and every column is
    compared by bubble index: indices exact, values within 1e-12 of each
    column's largest magnitude (columns that are differences of positions
    also within 4 ulp of the largest coordinate).
Both runs print 17 significant digits (--output-digits 17), which
round-trips a double; the default is the reference's 6.
"""
import ctypes as C
import os
import struct

import numpy as np
import pytest

from cubble_gb300 import _abi
from test_gpu_cli import results, run_cli, small_input

pytestmark = pytest.mark.gpu

DROWS = ["x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt", "dxdto", "dydto", "dzdto",
         "drdto", "path", "error", "saved_x", "saved_y", "saved_z", "saved_r"]
IROWS = ["wrap_count_x", "wrap_count_y", "wrap_count_z", "index", "num_neighbors"]


def read_checkpoint(path):
    """The checkpoint of cubble-cli (cli/cubble_cli.cpp write_checkpoint)."""
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:8] == b"CBGCKPT1"
    off = 8
    cfg = _abi.Config.from_buffer_copy(buf, off)
    off += C.sizeof(_abi.Config)
    rep = _abi.Report.from_buffer_copy(buf, off)
    off += C.sizeof(_abi.Report)
    (avg_rad, phi, time_scaling, e1, e2, snap_freq) = struct.unpack_from("<6d", buf, off)
    off += 48
    min_num, times_printed, num_snaps, add_flow = struct.unpack_from("<iIIi", buf, off)
    off += 16
    off += 24  # relative dimensions

    def vec(dtype):
        nonlocal off
        (n,) = struct.unpack_from("<Q", buf, off)
        off += 8
        a = np.frombuffer(buf, dtype=dtype, count=n, offset=off).copy()
        off += n * np.dtype(dtype).itemsize
        return a

    vec(np.int8)  # snapshot file name
    state = {k: vec(np.float64) for k in DROWS}
    state.update({k: vec(np.int32) for k in IROWS})
    pi, pj = vec(np.int32), vec(np.int32)
    prev = [vec(np.float64) for _ in range(3)]
    assert off == len(buf)
    return {"cfg": cfg, "report": rep.as_dict(), "avg_rad": avg_rad, "energy1": e1,
            "times_printed": times_printed, "num_snapshots": num_snaps,
            "add_flow": add_flow, "state": state, "pi": pi, "pj": pj, "prev": prev}


def oracle_from(oracle_mod, ck):
    o = oracle_mod.OracleFoam(ck["cfg"])
    o.load_state(ck["state"])
    o.set_pairs(ck["pi"], ck["pj"])
    r = ck["report"]
    o.set_time(r["time_step"], r["time_integer"], r["time_fraction"])
    o.set_options(1, ck["add_flow"], 1)  # simulate()'s options
    return o


@pytest.mark.parametrize("dim", [2, 3])
def test_cli_results_row_and_snapshot_match_oracle(tmp_path, oracle_mod, dim):
    a = os.path.join(str(tmp_path), "a")
    b = os.path.join(str(tmp_path), "b")
    os.makedirs(a)
    os.makedirs(b)
    over = {"snapShot.frequency": 1.0}
    if dim == 3:
        over["constants.phi.value"] = 0.8
    inp = small_input(dim=dim, num=2000 if dim == 2 else 3000, **over)
    run_cli(a, ["input.json", "--max-steps", "2500", "--checkpoint", "ck.bin",
                "--output-digits", "17"], inp)
    rows = results(a)
    assert len(rows) >= 2
    ck = read_checkpoint(os.path.join(a, "ck.bin"))
    s = ck["state"]
    n = ck["report"]["count"]
    row = rows[-1]
    # the row the checkpoint was written after
    assert row[0] == ck["times_printed"] - 1
    assert row[2] == n
    o = oracle_from(oracle_mod, ck)
    assert row[1] == pytest.approx(np.mean(s["r"]) / ck["avg_rad"], rel=1e-12)
    assert row[3] == pytest.approx(np.mean(s["path"]), rel=1e-12)
    assert row[4] == pytest.approx(o.energy(), rel=1e-12)
    assert ck["energy1"] == row[4]
    # dE from this row's and the previous row's energies (17 digits are exact)
    e, e_prev = row[4], rows[-2][4]
    de = abs(e - e_prev) * 2.0 / (e + e_prev) if e != e_prev else 0.0
    assert row[5] == pytest.approx(de, rel=1e-14)
    for c, k in ((6, "dxdt"), (7, "dydt"), (8, "dzdt"), (10, "drdt")):
        scale = max(float(np.mean(np.abs(s[k]))), 1e-300)
        assert abs(row[c] - np.mean(s[k])) <= 1e-12 * scale, k
    assert row[9] == pytest.approx(np.sqrt(row[6] ** 2 + row[7] ** 2 + row[8] ** 2), rel=1e-15)

    # one step on from the checkpoint: the resumed run's final snapshot
    run_cli(b, ["--resume", os.path.join(a, "ck.bin"), "--max-steps", "1",
                "--output-digits", "17"])
    written = sorted(int(f.rsplit(".", 1)[1]) for f in os.listdir(b)
                     if f.startswith("bubbles.csv."))
    assert written and written[0] == ck["num_snapshots"]
    # a snapshot time inside the step would write one more file first and move
    # the previous positions the final one's displacement is measured from
    check_disp = len(written) == 1
    snap = np.loadtxt(os.path.join(b, "bubbles.csv.%d" % written[-1]), delimiter=",",
                      skiprows=1, ndmin=2)
    o.integrate(1)
    so = o.get_state()
    eo = o.bubble_energies()
    cfg = ck["cfg"]
    iv = [cfg.tfr[q] - cfg.lbb[q] for q in range(3)]
    order = np.argsort(so["index"])
    idx = so["index"][order]
    got = snap[np.argsort(snap[:, 13])]
    assert np.array_equal(got[:, 13].astype(np.int64), idx)
    x, y, z = (so[k][order] for k in ("x", "y", "z"))
    vx, vy, vz = (so[k][order] for k in ("dxdt", "dydt", "dzdt"))
    disp = []
    for q, p in enumerate((x, y, z)):
        d = np.abs(p - ck["prev"][q][idx])
        disp.append(np.where(d > 0.5 * iv[q], d - iv[q], d))
    expect = {0: x - 0.5 * iv[0], 1: y - 0.5 * iv[1], 2: z - 0.5 * iv[2],
              3: so["r"][order], 4: vx, 5: vy, 6: vz,
              7: np.sqrt(vx * vx + vy * vy + vz * vz), 8: so["drdt"][order],
              9: so["path"][order], 10: eo[order],
              11: np.sqrt(disp[0] ** 2 + disp[1] ** 2 + disp[2] ** 2),
              12: so["error"][order]}
    ulp = 4.0 * float(np.spacing(max(float(np.max(np.abs(so[k]))) for k in ("x", "y", "z"))))
    for c, v in expect.items():
        if (dim == 2 and c in (2, 6)) or (c == 11 and not check_disp):
            continue
        diff = float(np.max(np.abs(got[:, c] - v)))
        allowed = 1e-12 * max(float(np.max(np.abs(v))), 1e-300)
        if c in (0, 1, 2, 9, 11, 12):  # positions and differences of positions
            allowed = max(allowed, ulp)
        assert diff <= allowed, (c, diff, allowed)

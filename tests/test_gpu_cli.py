"""GPU: cubble-cli, the drop-in for the reference's executable, end to end on
a small input: init (lattice, stabilisation, box rescale), the step loop
with results.dat rows and CSV snapshots, checkpoint / resume, array jobs."""
import json
import os
import subprocess

import numpy as np
import pytest

import cubble_gb300 as cb

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "cubble_gb300", "cubble-cli")


def small_input(dim=2, num=2000, **over):
    inp = {
        "bubbles": {"numStart": num, "numEnd": 200, "radius": {"mean": 1.0, "std": 0.21}},
        "box": {"dimensionality": dim, "relativeDimensions": {"x": 1.0, "y": 1.0, "z": 1.0},
                "wall": {"drag": 0.1, "x": 0, "y": 0, "z": 0}},
        "flow": {"impose": 0, "velocity": {"x": 0.01, "y": 0.0, "z": 0.0},
                 "lbb": {"x": 0.0, "y": 0.475, "z": 0.0},
                 "tfr": {"x": 0.4, "y": 0.525, "z": 0.0}},
        "constants": {"phi": {"value": 0.9}, "mu": {"value": 1.0}, "sigma": {"value": 1.0},
                      "kappa": {"value": 0.1}, "K": {"value": 2.0}},
        "errorTolerance": {"value": 1e-5},
        "rngSeed": {"value": 426},
        "stabilization": {"steps": 200, "maxDeltaEnergy": 10.0},
        "snapShot": {"filename": "bubbles", "frequency": 0.0},
    }
    for path, v in over.items():
        d = inp
        keys = path.split(".")
        for k in keys[:-1]:
            d = d[k]
        d[keys[-1]] = v
    return inp


def run_cli(tmp, args, inp=None):
    cb.build()
    assert os.path.exists(CLI), "cubble-cli was not built"
    if inp is not None:
        with open(os.path.join(tmp, "input.json"), "w") as f:
            json.dump(inp, f)
    p = subprocess.run([CLI] + args, cwd=tmp, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    return p.stdout


def results(tmp):
    rows = np.loadtxt(os.path.join(tmp, "results.dat"), ndmin=2)
    assert rows.shape[1] == 11
    return rows


def test_cli_runs_and_writes_outputs(tmp_path):
    tmp = str(tmp_path)
    out = run_cli(tmp, ["input.json", "--max-steps", "4000"],
                  small_input(**{"snapShot.frequency": 2.0}))
    assert "Stabilization" in out and "Integration" in out
    rows = results(tmp)
    assert len(rows) >= 2
    assert np.array_equal(rows[:, 0], np.arange(1, len(rows) + 1))  # printed time units
    assert np.all(np.diff(rows[:, 2]) <= 0)       # bubble count never grows
    assert np.all(np.isfinite(rows))
    assert np.all(rows[:, 1] > 0.9)               # <r> / r0 grows by coarsening
    snaps = sorted(f for f in os.listdir(tmp) if f.startswith("bubbles.csv."))
    assert len(snaps) >= 3
    with open(os.path.join(tmp, snaps[0])) as f:
        head = f.readline().strip()
    assert head == "x,y,z,r,vx,vy,vz,vtot,vr,path,energy,displacement,error,index"
    data = np.loadtxt(os.path.join(tmp, snaps[-1]), delimiter=",", skiprows=1, ndmin=2)
    assert data.shape[1] == 14 and np.all(np.isfinite(data))
    assert len(np.unique(data[:, 13])) == len(data)  # bubble indices are unique


def test_cli_mixed_form_and_3d(tmp_path):
    tmp = str(tmp_path)
    inp = small_input(dim=3, num=3000, **{"constants.phi.value": 0.8})
    inp["gb300"] = {"precision": "mixed"}
    out = run_cli(tmp, ["input.json", "--max-steps", "1500"], inp)
    assert "mixed form" in out
    assert len(results(tmp)) >= 1


def test_cli_fp64_ff_form_matches_fp64(tmp_path):
    """--precision fp64_ff (pair terms in float-float) against the default
    FP64 form on the same input: the first printed rows agree to 1e-9."""
    rows = {}
    for form in ("fp64", "fp64_ff"):
        tmp = os.path.join(str(tmp_path), form)
        os.makedirs(tmp)
        out = run_cli(tmp, ["input.json", "--max-steps", "800", "--precision", form],
                      small_input())
        assert ("%s form" % form) in out
        rows[form] = results(tmp)
    k = min(len(rows["fp64"]), len(rows["fp64_ff"]), 2)
    assert k >= 1
    np.testing.assert_allclose(rows["fp64_ff"][:k], rows["fp64"][:k], rtol=1e-9, atol=1e-12)


def test_cli_walls_and_shear_3d(tmp_path):
    """3D with walls in z and the linear shear extension (the large sheared
    foam's setting), mixed form: runs, writes finite rows, and the mean x
    velocity of the snapshot grows with height (the imposed profile)."""
    tmp = str(tmp_path)
    inp = small_input(dim=3, num=3000, **{"constants.phi.value": 0.8, "box.wall.z": 1,
                                          "flow.impose": 1, "snapShot.frequency": 1.0})
    inp["gb300"] = {"precision": "mixed", "shear": 0.05}
    run_cli(tmp, ["input.json", "--max-steps", "1500"], inp)
    rows = results(tmp)
    assert np.all(np.isfinite(rows))
    snaps = sorted((f for f in os.listdir(tmp) if f.startswith("bubbles.csv.")),
                   key=lambda f: int(f.rsplit(".", 1)[1]))
    data = np.loadtxt(os.path.join(tmp, snaps[-1]), delimiter=",", skiprows=1, ndmin=2)
    z, vx = data[:, 2], data[:, 4]
    lo, hi = z < np.quantile(z, 0.25), z > np.quantile(z, 0.75)
    assert vx[hi].mean() - vx[lo].mean() > 0.02


def test_cli_checkpoint_resume_continues(tmp_path):
    a = os.path.join(str(tmp_path), "a")
    b = os.path.join(str(tmp_path), "b")
    os.makedirs(a)
    os.makedirs(b)
    inp = small_input()
    run_cli(a, ["input.json", "--max-steps", "6000"], inp)
    full = results(a)
    assert len(full) >= 4
    os.makedirs(os.path.join(a, "first"))
    first = os.path.join(a, "first")
    run_cli(first, ["../input.json", "--max-steps", "2500", "--checkpoint", "ck.bin"])
    part = results(first)
    k = len(part)
    assert 1 <= k < len(full)
    # the run to the checkpoint equals the start of the uninterrupted run
    np.testing.assert_allclose(part, full[:k], rtol=1e-6, atol=1e-12)
    steps_to_ck = None
    out = run_cli(b, ["--resume", os.path.join(first, "ck.bin"), "--max-steps", "3000"])
    assert "Resumed" in out
    cont = results(b)
    assert cont[0, 0] == k + 1
    m = min(len(cont), len(full) - k)
    assert m >= 1
    np.testing.assert_allclose(cont[:m], full[k:k + m], rtol=1e-6, atol=1e-12)
    del steps_to_ck


def test_cli_profile_range_keeps_results(tmp_path):
    """--profile-range (the reference's PROFILE option: the profiler's capture
    range over the first stretch of the step loop) ends the graph stretches
    at its stop step and changes nothing else: results.dat matches the run
    without it to the rounding of the FP64 reductions (whose order is free
    from run to run)."""
    a = os.path.join(str(tmp_path), "a")
    b = os.path.join(str(tmp_path), "b")
    os.makedirs(a)
    os.makedirs(b)
    inp = small_input()
    run_cli(a, ["input.json", "--max-steps", "2500", "--output-digits", "17"], inp)
    run_cli(b, ["input.json", "--max-steps", "2500", "--output-digits", "17", "--profile-range"],
            inp)
    ra, rb = results(a), results(b)
    assert ra.shape == rb.shape and len(ra) >= 2
    np.testing.assert_allclose(rb, ra, rtol=1e-9, atol=1e-12)


def test_cli_array_jobs(tmp_path):
    tmp = str(tmp_path)
    with open(os.path.join(tmp, "array.params"), "w") as f:
        f.write("two jobs\n{\n    constants.phi.value = 0.92\n    bubbles.numStart = 1500\n}\n"
                "{\n    constants.phi.value = 0.88\n}\n")
    out = run_cli(tmp, ["input.json", "--array", "array.params", "--max-steps", "800"],
                  small_input())
    assert "array job 2 of 2" in out
    for k in (0, 1):
        assert os.path.exists(os.path.join(tmp, "run_%d" % k, "results.dat"))

"""CPU tests of the C-ABI boundary: the library loads, exports every entry
point include/cubble_gb300.h declares, its structures have the C layout, and
without a usable GPU it fails loudly instead of falling back."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

import cubble_gb300 as cb
from cubble_gb300 import _abi
from cubble_gb300.foam import CubbleError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = cb.lib()
    declared = cb.exported_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", cb.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported
    # nothing but the C ABI is exported from the product library
    assert {s for s in exported if s.startswith("cb_")} == set(declared)


def _c_layout():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "cubble_gb300.h"
#define P(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))
int main(void) {
  printf("cb_config %zu\ncb_state_view %zu\ncb_report %zu\ncb_attempt_view %zu\n",
         sizeof(cb_config), sizeof(cb_state_view), sizeof(cb_report), sizeof(cb_attempt_view));
  P(cb_config, lbb); P(cb_config, time_step); P(cb_config, use_graph);
  P(cb_state_view, x); P(cb_state_view, num_neighbors);
  P(cb_report, time_fraction); P(cb_report, status);
  P(cb_attempt_view, delete_flags); P(cb_attempt_view, num_to_be_deleted);
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        with open(c, "w") as f:
            f.write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return dict((ln.split()[0], int(ln.split()[1])) for ln in out.splitlines())


def test_struct_layouts_match_c():
    lay = _c_layout()
    assert lay["cb_config"] == C.sizeof(_abi.Config)
    assert lay["cb_state_view"] == C.sizeof(_abi.StateView)
    assert lay["cb_report"] == C.sizeof(_abi.Report)
    assert lay["cb_attempt_view"] == C.sizeof(_abi.AttemptView)
    for key, val in lay.items():
        if "." not in key:
            continue
        t, f = key.split(".")
        cls = {"cb_config": _abi.Config, "cb_state_view": _abi.StateView,
               "cb_report": _abi.Report, "cb_attempt_view": _abi.AttemptView}[t]
        assert getattr(cls, f).offset == val, key


def test_invalid_configuration_is_rejected(gpu_lib):
    cfg = cb.make_config(dimensionality=4, capacity=10)
    with pytest.raises(CubbleError) as e:
        cb.GpuFoam(cfg)
    assert e.value.code in (_abi.CB_ERR_INVALID_ARGUMENT, _abi.CB_ERR_NO_DEVICE)


@pytest.mark.parametrize("dim,capacity,pair_capacity,ok", [
    (3, 134_000_000, 0, True),         # default 16 per bubble: 2.14e9 pairs
    (3, 135_000_000, 0, False),        # default would pass 2^31 - 2
    (3, 135_000_000, 1_500_000_000, True),
    (2, 268_000_000, 0, True),         # default 8 per bubble in 2D
    (2, 10, -1, False),
    (2, 10, 2_147_483_647, False),
])
def test_pair_capacity_range(gpu_lib, dim, capacity, pair_capacity, ok):
    """Configuration checks run before the device is touched: a pair list
    that int32 offsets cannot address is rejected on any machine."""
    import torch
    cfg = cb.make_config(dimensionality=dim, capacity=capacity, pair_capacity=pair_capacity)
    if ok and torch.cuda.is_available():
        pytest.skip("would allocate the full capacity")
    with pytest.raises(CubbleError) as e:
        cb.GpuFoam(cfg)
    want = _abi.CB_ERR_NO_DEVICE if ok else _abi.CB_ERR_INVALID_ARGUMENT
    assert e.value.code == want, cb.lib().cb_last_error()


def test_no_device_fails_loudly(gpu_lib):
    """With no GPU the product raises; it never computes on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cfg = cb.make_config(dimensionality=2, capacity=10)
    with pytest.raises(CubbleError) as e:
        cb.GpuFoam(cfg)
    assert e.value.code == _abi.CB_ERR_NO_DEVICE

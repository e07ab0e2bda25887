"""The ray kernel's stream precision.  The default (MRF_PRECISION_FP32) reads
segment lengths and gathers ln q as fp32; MRF_PRECISION_HALF_STREAMS reads
both as fp16, with every product, prefix and sum in fp32 (fp64 on long rays)
and fp32 messages.  Both are measured against the FP64 oracle on the small
room (Gauss-Seidel and Jacobi, 10 iterations): the default at the tests'
belief tolerance (1e-3, >= 99.9 % class agreement), the 16-bit streams at
the bound they are documented with (1e-2; measured 2.6e-3 Gauss-Seidel,
4.5e-3 Jacobi, which is why they are not the default).  Switching back to
the default reproduces it bit for bit.  The errors are printed for the
record."""
import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [0, L.JACOBI], ids=["gauss-seidel", "jacobi"])
def test_stream_precisions_against_oracle(native_lib, oracle_lib, small_room, flags):
    w = small_room
    gm = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(w.params, threads=8)
    for P, D in zip(w.poses, w.depths):
        gm.add_view(P, D)
        om.add_view(P, D, O.ACT_FULL_RAY)
    om.infer(flags=O.JACOBI if flags else 0)
    ob = om.beliefs()
    gm.infer(flags=flags)
    b32 = gm.beliefs()
    gm.set_precision(L.PRECISION_HALF_STREAMS)
    gm.reset_state()
    gm.infer(flags=flags)
    b16 = gm.beliefs()
    for name, b, tol in (("fp32 streams (default)", b32, 1e-3), ("fp16 streams", b16, 1e-2)):
        b = b.astype(np.float64)
        touched = (b > 0) | (ob > 0)
        err = np.abs(b - ob).max()
        agree = ((b > 0.5) == (ob > 0.5))[touched].mean()
        print(f"{name}: max belief error {err:.3e}, class agreement {agree:.6f}")
        assert err <= tol and agree >= 0.999
    gm.set_precision(L.PRECISION_FP32)
    gm.reset_state()
    gm.infer(flags=flags)
    np.testing.assert_array_equal(gm.beliefs(), b32)
    with pytest.raises(L.MrfError):
        gm.set_precision(7)
    gm.close()
    om.close()

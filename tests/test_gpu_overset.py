"""GPU parity of the overset interpolation (src/connectivity.f:2-190)
through the C-ABI drop-in ot2d_do_interpolations: seeded multi-mesh
systems with random donor / fringe lists (one fringe cell listed twice, so
the later entry must win), Euler / SA / SST variable sets, one and three
time instances, host arrays and device-resident q, against the oracle.

Tolerance: bit-exact -- the gather keeps the reference's weights and term
order and the FP64 kernels are compiled without fused multiply-adds."""
import numpy as np
import pytest

from tests import oracle_binding as ob
from tests.overset_case import make_params, make_system, oracle_interp
from turns2d_urans_git_gb300 import routines as rt

pytestmark = pytest.mark.gpu


def _args(d, qg):
    return (qg, d["jmx"], d["kmx"], d["ibcg"], d["imeshg"], d["idonorg"], d["fracg"], d["nfringeg"], d["ndonorg"],
            d["iisptrg"], d["iieptrg"], d["idsize"], d["qsize"], d["nmesh"])


@pytest.mark.parametrize("iturb,nspec", [(0, 1), (1, 1), (2, 1), (1, 3)])
def test_do_interpolations_matches_oracle(iturb, nspec):
    p = make_params(nspec, iturb)
    d = make_system(p, 40 + 3 * iturb + nspec)
    q_o = oracle_interp(ob.lib(), ob.ptr, p, d)
    assert not np.array_equal(q_o, d["qg"])
    rt.set_params(p)
    qg = d["qg"].copy()
    rt.do_interpolations(*_args(d, qg))
    assert np.array_equal(qg, q_o)


def test_do_interpolations_device_resident():
    torch = pytest.importorskip("torch")
    p = make_params(1, 1)
    d = make_system(p, 77)
    q_o = oracle_interp(ob.lib(), ob.ptr, p, d)
    rt.set_params(p)
    qd = torch.from_numpy(d["qg"].copy()).cuda()
    rt.do_interpolations(*_args(d, qd))
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), q_o)


def test_do_interpolations_rejects_stencil_outside_mesh():
    p = make_params(1, 1)
    d = make_system(p, 78)
    d["idonorg"][0, 0, 0, 0] = 1          # stencil would read column 0
    rt.set_params(p)
    qg = d["qg"].copy()
    with pytest.raises(rt.RoutineError) as e:
        rt.do_interpolations(*_args(d, qg))
    assert e.value.code == 1
    assert np.array_equal(qg, d["qg"])    # nothing written

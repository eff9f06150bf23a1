"""Error behaviour of the C ABI: invalid configurations are refused with
the reference's messages (PARTHENON_THROW/REQUIRE in fluid.cpp), an
unbracketed con2prim root is reported on the next check (the reference
aborts, root_find.hpp:115-118), and calls that need state that was never
set (the learned start without weights) are refused."""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from phoebus_gb300.abi import PhxError

pytestmark = pytest.mark.gpu


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_invalid_params_refused(ctx_fast):
    b = states.random_block(8, states.SEED + 61).to_device("cuda")
    for over, msg in ((dict(recon=7), "invalid recon"), (dict(riemann=9), "invalid riemann"),
                      (dict(c2p_floor_scale_fac=0.0), "c2p_floor_scale_fac must be between 0 and 1"),
                      (dict(c2p_max_iter=-1), "c2p_max_iter")):
        p = abi.default_params(**over)
        with pytest.raises(PhxError) as e:
            ctx_fast.CalculateFluxes(p, b)
        assert e.value.status == 1 and msg in str(e.value), str(e.value)


def test_invalid_block_refused(ctx_fast):
    hb = states.random_block(8, states.SEED + 62)
    b = hb.to_device("cuda")
    b.ng = 2  # the stencils need three ghost layers
    with pytest.raises(PhxError) as e:
        ctx_fast.CalculateFluxes(abi.default_params(), b)
    assert e.value.status == 1 and "ng must be >= 3" in str(e.value)


def test_zone_calls_refuse_bad_sizes_and_missing_weights(built):
    import torch

    from phoebus_gb300.fluid import FluidContext

    ctx = FluidContext(0, exact=False)  # fresh: no learned weights loaded
    try:
        p = abi.default_params()
        cons = torch.zeros((abi.NCONS, 64), dtype=torch.float64, device="cuda")
        prim = torch.zeros((abi.NPRIM, 64), dtype=torch.float64, device="cuda")
        with pytest.raises(PhxError) as e:
            ctx.ConservedToPrimitiveZones(p, cons, prim, learned=True)
        assert e.value.status == 1 and "no learned-guess weights" in str(e.value)
        with pytest.raises(PhxError) as e:
            ctx.MLPForward(torch.zeros((6, 8), dtype=torch.float32, device="cuda"))
        assert e.value.status == 1
        with pytest.raises(PhxError) as e:
            ctx.MLPTrain(torch.zeros((6, 8), dtype=torch.float32, device="cuda"),
                         torch.zeros(8, dtype=torch.float32, device="cuda"))
        assert e.value.status == 1 and "smaller than one batch" in str(e.value)
        with pytest.raises(PhxError) as e:
            ctx.MLPTrain(torch.zeros((6, 8192), dtype=torch.float32, device="cuda"),
                         torch.zeros(8192, dtype=torch.float32, device="cuda"),
                         abi.default_train_opts(epochs=abi.MLP_MAX_EPOCHS + 1))
        assert e.value.status == 7
        ctx.check()
    finally:
        ctx.close()


def test_unbracketed_root_reported(ctx_exact, oracle):
    """tau = -0.9 D with no momentum or field: f(0) and f(1) are both
    negative, the root is not bracketed.  The zone keeps its guess, its fail
    flag is 0, and the next check raises the reference's abort message."""
    n = 64
    prim = np.zeros((abi.NPRIM, n))
    prim[abi.PRHO] = 1.0
    prim[abi.PENG] = 0.5
    prim[abi.PPRS] = 0.5 / 3.0
    prim[abi.PGM1] = 4.0 / 3.0
    prim[abi.PTMP] = 0.5
    cons = oracle.PrimitiveToConservedZones(abi.default_params(), prim)
    cons[abi.CENG, 17] = -0.9 * cons[abi.CRHO, 17]
    p = abi.default_params()
    rfail = np.zeros(n)
    unbr = oracle.ConservedToPrimitiveZones(p, cons.copy(), prim.copy(), fail=rfail)
    assert unbr == 1 and rfail[17] == 0.0
    c, pr = dev(cons), dev(prim)
    fail = ctx_exact.ConservedToPrimitiveZones(p, c, pr)
    with pytest.raises(PhxError) as e:
        ctx_exact.check()
    assert e.value.status == 2 and "Aborting with unbracketed root." in str(e.value)
    f = fail.cpu().numpy()
    assert f[17] == 0.0 and f.sum() == n - 1
    ctx_exact.check()  # the sticky word was cleared by the report

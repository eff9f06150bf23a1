"""Error behaviour of the C ABI: invalid configurations are refused with
the reference's messages (PARTHENON_THROW/REQUIRE in fluid.cpp), and calls
that need state that was never set (the learned start without weights) or
exceed a fixed capacity are refused.  (An unbracketed con2prim root, which
the reference aborts on, cannot be produced from finite inputs: the robust
residual with the EOS floor sie >= 0 always changes sign on [0, 1].)"""
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


def test_bounded_wait_times_out_and_context_recovers(built):
    """The bounded-wait failure path, driven in the allowed form: a thread
    block arms an mbarrier for bytes that no copy will deliver (nothing in
    flight), gives up after 1000 polls, sets the timeout bit and returns.
    phx_ctx_check reports PHX_ERR_TIMEOUT once; afterwards the same context
    runs the bulk-copy flux kernel (the same wait) and checks clean, and
    another context was never affected."""
    from phoebus_gb300.fluid import FluidContext

    ctx, other = FluidContext(0, exact=False), FluidContext(0, exact=False)
    try:
        assert ctx.lib.phx_probe_bounded_wait(ctx.h, 0, None) == abi.PHX_ERR_INVALID_ARG
        assert ctx.lib.phx_probe_bounded_wait(ctx.h, 1000, None) == abi.PHX_OK
        with pytest.raises(PhxError) as e:
            ctx.check()
        assert e.value.status == abi.PHX_ERR_TIMEOUT and "bounded device wait" in str(e.value)
        ctx.check()  # the bit was cleared
        other.check()
        p = abi.default_params(Gamma=5.0 / 3.0, recon="weno5z", riemann="hll")
        hb, _ = states.kelvin_helmholtz(n=12, seed=11)
        b = hb.to_device("cuda")
        ctx.Initialize(p, b)
        ctx.CalculateFluxes(p, b)
        ctx.check()
        import torch

        assert bool(torch.isfinite(b["flux"][:, 4:17, 4:17, 4:17]).all())
    finally:
        ctx.close()
        other.close()

"""GPU: the host-buffer forms (grns_div_host, grns_scale2pow_host) give the
results of the device-pointer forms for every chunking, layout and kind of
host memory."""
import numpy as np
import pytest

from grns_gb300 import workload as W
from oracle import oracle as O
from tests.helpers import moduli_for

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", params=["g8", "g32", "p64"])
def case(request):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import grns_gb300 as G
    mods = moduli_for(request.param)
    return G.RNSContext(mods), O.Oracle(mods)


def host(a, layout, pinned):
    t = torch.from_numpy(np.ascontiguousarray(a if layout == "aos" else a.T, dtype=np.int32))
    return t.pin_memory() if pinned else t


@pytest.mark.parametrize("layout", ["soa", "aos"])
@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("chunks", [0, 1, 3, 7])
def test_div_host(case, layout, pinned, chunks):
    ctx, orc = case
    N = 20001
    x = W.uniform_residues(orc.moduli, N, seed=3, stream=W.S_X, layout="aos")
    d, _ = W.divisors(orc.moduli, orc.log2M, N, seed=3, layout="aos")
    d[5] = 0  # a zero divisor: flagged, q = 0, r = x
    hx, hd = host(x, layout, pinned), host(d, layout, pinned)
    flags = torch.zeros(N, dtype=torch.uint8, pin_memory=pinned)
    q, r = ctx.rns_div_host(hx, hd, layout=layout, flags=flags, chunks=chunks)
    torch.cuda.current_stream().synchronize()
    dflags = torch.zeros(N, dtype=torch.uint8, device="cuda")
    qd, rd = ctx.rns_div(hx.cuda(), hd.cuda(), layout=layout, flags=dflags)
    assert torch.equal(q, qd.cpu()) and torch.equal(r, rd.cpu())
    assert torch.equal(flags, dflags.cpu()) and int(flags[5]) == 2


@pytest.mark.parametrize("layout", ["soa", "aos"])
@pytest.mark.parametrize("chunks", [0, 2, 5])
def test_scale2pow_host(case, layout, chunks):
    ctx, orc = case
    N = 30011
    x = W.uniform_residues(orc.moduli, N, seed=4, stream=W.S_X, layout="aos")
    D = torch.from_numpy((np.arange(N, dtype=np.int64) * 37 % (orc.log2M + 3)).astype(np.int32)).pin_memory()
    hx = host(x, layout, True)
    out = ctx.rns_scale2pow_host(hx, D, layout=layout, chunks=chunks)
    torch.cuda.current_stream().synchronize()
    ref = ctx.rns_scale2pow(hx.cuda(), D.cuda(), layout=layout)
    assert torch.equal(out, ref.cpu())
    out = ctx.rns_scale2pow_host(hx, 77, layout=layout, chunks=chunks)
    torch.cuda.current_stream().synchronize()
    assert torch.equal(out, ctx.rns_scale2pow(hx.cuda(), 77, layout=layout).cpu())


def test_host_forms_order_on_the_stream(case):
    """results are complete when the caller's stream reaches the call's end"""
    ctx, orc = case
    N = 4096
    x = host(W.uniform_residues(orc.moduli, N, seed=5, stream=W.S_X, layout="aos"), "soa", True)
    s = torch.cuda.Stream()
    q, r = ctx.rns_div_host(x, x, stream=s, chunks=4)
    s.synchronize()
    assert orc.exact.from_rns(q.numpy().T) == [1 if v else 0 for v in orc.exact.from_rns(x.numpy().T)]
    assert not r.any()

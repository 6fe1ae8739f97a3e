"""gbpf_batch_solve_noalloc, the entry point that allocates nothing, against
the allocating batch entry points on the same instances, two calls in a row.

Who needs it: callers that cannot allocate device memory when they solve --
a real-time loop with a fixed cycle time, where cudaMalloc (which can
synchronise the device and takes an unbounded time) is not allowed after
start-up, or code inside a host framework whose device memory belongs to that
framework's allocator.  The entry point works on their device buffers and
keeps its own scratch in one static 8 MiB device array.  It runs every
instance on the block-per-instance kernel, while the allocating path serves
these small grids with the warp-per-instance kernel; the two sum the LU
updates of a pivot in different orders, so the results agree to rounding.
FP64: |V| and theta to 1e-12, the final mismatch (itself ~1e-13) to 1e-12
absolute, iteration counts and statuses exactly.  FP32 LU (FP64 mismatch,
test and update): statuses exactly, iterations within one, |V| and theta to
1e-6 (the tolerance the other FP32 batch tests hold), final mismatch <= 1e-8.
The second call uses other instances, so stale contents of the shared scratch
would show up, and the device's free memory must not change across it.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ieee_cases, ieee_path

pytestmark = pytest.mark.gpu


def _instances(grids, n, seed):
    rng = np.random.default_rng(seed)
    gi = rng.integers(0, len(grids), n).astype(np.int32)
    cols = {k: [] for k in ("Pload", "Qload", "Pg", "Qg", "V0", "theta0")}
    for t in gi:
        b = grids[t].buses()
        lf = np.exp(rng.normal(-0.005, 0.1, grids[t].nB))
        gf = rng.uniform(0.9, 1.1, grids[t].nB)
        cols["Pload"].append(b["Pload"] * lf)
        cols["Qload"].append(b["Qload"] * lf)
        cols["Pg"].append(b["Pg"] * gf)
        cols["Qg"].append(b["Qg"])
        cols["V0"].append(b["V0"])
        cols["theta0"].append(b["theta0"])
    return gi, {k: np.concatenate(v) for k, v in cols.items()}


@pytest.mark.parametrize("precision", ["PREC_FP64", "PREC_FP32_IR"])
def test_noalloc_matches_batch_on_two_calls(gb, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    grids = [gb.read_grid(os.path.join(GOLDEN, "c1.cdf")), gb.read_grid(os.path.join(GOLDEN, "c2_base.cdf"))]
    opts = dict(tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1, precision=getattr(gb, precision))
    fp64 = precision == "PREC_FP64"
    noalloc = gb.Batch(grids, **opts)
    reference = gb.Batch(grids, **opts)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call, (n, seed) in enumerate(((24, 1), (37, 2))):
        gi, c = _instances(grids, n, seed)
        reference.set_instances(gi, Pload=c["Pload"], Qload=c["Qload"], Pg=c["Pg"], Qg=c["Qg"], V0=c["V0"],
                                theta0=c["theta0"])
        reference.solve()
        ref = reference.results()
        t = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
        V0, th0 = t(c["V0"]), t(c["theta0"])
        Pliq, Qliq, Qload = t(c["Pg"] - c["Pload"]), t(c["Qg"] - c["Qload"]), t(c["Qload"])
        nb = len(c["V0"])
        V, th, P, Q = (torch.full((nb,), float("nan"), dtype=torch.float64, device=dev) for _ in range(4))
        it = torch.full((n,), -1, dtype=torch.int32, device=dev)
        st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        mm = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        free0 = torch.cuda.mem_get_info(dev)[0]
        noalloc.solve_noalloc(gi, V0.data_ptr(), th0.data_ptr(), Pliq.data_ptr(), Qliq.data_ptr(), Qload.data_ptr(),
                              V.data_ptr(), th.data_ptr(), P.data_ptr(), Q.data_ptr(), it.data_ptr(), st.data_ptr(),
                              mm.data_ptr(), stream=stream.cuda_stream)
        torch.cuda.synchronize(dev)
        if call == 1:  # the first call may load the kernel's module; the second allocates nothing at all
            assert torch.cuda.mem_get_info(dev)[0] == free0
        np.testing.assert_array_equal(st.cpu().numpy(), ref["status"])
        if fp64:
            np.testing.assert_array_equal(it.cpu().numpy(), ref["iterations"])
            assert np.max(np.abs(V.cpu().numpy() - ref["V"])) <= 1e-12
            assert np.max(np.abs(th.cpu().numpy() - ref["theta"])) <= 1e-12
            assert np.max(np.abs(P.cpu().numpy() - ref["Pcalc"])) <= 1e-10
            np.testing.assert_allclose(mm.cpu().numpy(), ref["final_mismatch"], rtol=0, atol=1e-12)
        else:
            assert np.max(np.abs(it.cpu().numpy() - ref["iterations"])) <= 1
            assert np.max(np.abs(V.cpu().numpy() - ref["V"])) <= 1e-6
            assert np.max(np.abs(th.cpu().numpy() - ref["theta"])) <= 1e-6
        assert np.all(mm.cpu().numpy()[st.cpu().numpy() == 0] <= 1e-8)


def test_noalloc_rejects_a_grid_beyond_shared_memory(gb):
    """A 3,776-bus grid's state does not fit one block's shared memory: the
    call says so (GBPF_E_ARG) instead of failing in the launch."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    case = next(c for c in ieee_cases() if c["cdf"] == "ieee118x32.cdf")
    grids = [gb.read_grid(os.path.join(GOLDEN, "c1.cdf")), gb.read_grid(ieee_path(case))]
    b = gb.Batch(grids, tolerancia=1e-8, no_max_iter=100)
    x = torch.zeros(4 * 3776, dtype=torch.float64, device="cuda")
    with pytest.raises(gb.GbpfError) as e:
        b.solve_noalloc(np.array([0, 1], np.int32), *([x.data_ptr()] * 9), x.data_ptr(), x.data_ptr(),
                        x.data_ptr())
    assert e.value.status == gb.E_ARG
    assert "shared memory" in str(e.value)


def test_noalloc_rejects_too_many_instances(gb):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    grid = gb.read_grid(os.path.join(GOLDEN, "c1.cdf"))
    b = gb.Batch([grid], tolerancia=1e-8, no_max_iter=100)
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    n = 600000  # metadata alone exceeds the static scratch
    with pytest.raises(gb.GbpfError) as e:
        b.solve_noalloc(np.zeros(n, np.int32), *([x.data_ptr()] * 9), x.data_ptr(), x.data_ptr(), x.data_ptr())
    assert e.value.status == gb.E_ARG
    assert "static scratch" in str(e.value)

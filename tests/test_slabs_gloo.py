"""Depth-slab decomposition with a per-step halo exchange, on CPU: two gloo ranks each run the FP64
oracle on their slab and exchange the overlap rows of every state field over torch.distributed
after every step; the gathered traces equal the single-domain oracle's exactly. Plus the host-side
layout, slicing and exchange plan."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _problem():
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(48, 40), nt=70, n_pml=8, n_transition=8)
    rng = np.random.default_rng(3)
    # sensors on every depth row of a column (some in each slab), air cells near the cut
    nx, ny = inp.shape
    inp.outc = np.stack([np.arange(8, nx - 8), np.full(nx - 16, ny // 2)], 1).astype(np.int32)
    inp.icczero = np.stack([rng.integers(30, 60, 20), rng.integers(8, ny - 8, 20)], 1).astype(np.int32)
    return inp


def _state_arrays(oracle):
    st = oracle.state
    out = [st.p] + list(st.v)
    for a in range(len(st.v)):
        out += [st.psi[a][0], st.psi[a][1]]
    for a in range(len(st.v)):
        out += [st.phi[a][0], st.phi[a][1]]
    return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    from fdtd_oracle import Oracle
    from fullwave25_gb300.slabs import OVERLAP, exchanges, slab_layout, slice_inputs

    inp = _problem()
    slabs = slab_layout(inp.shape[0], world)
    part, idx = slice_inputs(inp, slabs[rank])
    orc = Oracle(part)
    traces = np.zeros((inp.n_out, idx.size))
    plan = exchanges(slabs, OVERLAP)
    for _ in range(inp.nt):
        orc.step(traces)
        arrays = _state_arrays(orc)
        reqs, recv = [], []
        for dst, drow, src, srow, n in plan:
            if src == rank:
                buf = torch.from_numpy(np.stack([a[srow:srow + n] for a in arrays]).copy())
                reqs.append(dist.isend(buf, dst))
            if dst == rank:
                buf = torch.empty((len(arrays), n) + arrays[0].shape[1:], dtype=torch.float64)
                reqs.append(dist.irecv(buf, src))
                recv.append((drow, n, buf))
        for r in reqs:
            r.wait()
        for drow, n, buf in recv:
            for a, b in zip(arrays, buf.numpy()):
                a[drow:drow + n] = b
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx.tolist(), traces))
    out.put((rank, gathered))
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_single_domain_oracle():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
    from fdtd_oracle import run_oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    inp = _problem()
    ref = run_oracle(inp)
    got = np.zeros_like(ref)
    _, gathered = res[0]
    covered = 0
    for idx, tr in gathered:
        got[:, idx] = tr
        covered += len(idx)
    assert covered == ref.shape[1]
    assert np.abs(ref).max() > 0
    np.testing.assert_array_equal(got, ref)


def test_layout_and_exchange_plan():
    from fullwave25_gb300.slabs import exchanges, slab_layout

    slabs = slab_layout(200, 3, overlap=16)
    assert slabs[0].own[0] == 8 and slabs[-1].own[1] == 192
    assert slabs[0].dom == (0, slabs[0].own[1] + 24) and slabs[-1].dom[1] == 200
    for a, b in zip(slabs, slabs[1:]):
        assert a.own[1] == b.own[0]
    plan = exchanges(slabs, 16)
    assert len(plan) == 4
    dst, drow, src, srow, n = plan[0]
    assert (dst, src, n) == (0, 1, 16)
    # the copied rows are the same global rows on both sides
    assert slabs[dst].dom[0] + drow == slabs[src].dom[0] + srow == slabs[0].own[1]
    with pytest.raises(ValueError):
        slab_layout(200, 3, overlap=8)
    with pytest.raises(ValueError):
        slab_layout(60, 4, overlap=16)


def test_slice_keeps_sources_in_grid_and_sensors_owned():
    from fullwave25_gb300.slabs import slab_layout, slice_inputs

    inp = _problem()
    slabs = slab_layout(inp.shape[0], 2)
    seen = []
    for s in slabs:
        part, idx = slice_inputs(inp, s)
        assert part.shape == (s.dom[1] - s.dom[0], inp.shape[1])
        rows = inp.outc[idx, 0]
        assert ((rows >= s.own[0]) & (rows < s.own[1])).all()
        assert part.icc.shape[0] == part.icmat.shape[0]
        np.testing.assert_array_equal(part.maps["rho"], inp.maps["rho"][s.dom[0]:s.dom[1]])
        seen += idx.tolist()
    assert sorted(seen) == list(range(inp.outc.shape[0]))

"""The serving loop: admission under an HBM budget, LRU eviction, continuous
batching, and the same result alone and in the mix."""
import pytest
import torch

import oracle
import tron_grid_gb300 as tg
from tron_grid_gb300 import scene
from tron_grid_gb300.batch import Batch
from tron_grid_gb300.serve import Server

pytestmark = pytest.mark.gpu
KEYS = ("radiance", "depth", "normal", "motion")


def _host_seq(w, h, frames, seed, f16=False, pinned=True):
    sc = scene.PlaneScene(scene.pan_with_disocclusion(w, h, seed=seed))
    seq = []
    for t in range(frames):
        fr = sc.frame(t)
        d = {k: fr[k] for k in KEYS}
        if f16:
            d["radiance"] = d["radiance"].half()
            d["normal"] = torch.from_numpy(oracle.oct16_encode(fr["normal"].numpy()))
        seq.append({k: (v.contiguous().pin_memory() if pinned else v.contiguous().clone()) for k, v in d.items()})
    return seq


def _single(w, h, seq, storage, dev):
    d = tg.Denoiser(w, h, storage=storage)
    dt = torch.float16 if storage == tg.STORAGE_FP16 else torch.float32
    outs = []
    for fr in seq:
        o = torch.empty((h, w, 4), dtype=dt, device=dev)
        d.denoise(*(fr[k].to(dev) for k in KEYS), out=o)
        outs.append(o.cpu())
    d.close()
    return outs


@pytest.mark.parametrize("batching,strategy,pinned", [(True, 0, True), (True, 1, True), (False, 0, True),
                                                      (True, 0, False), (False, 0, False)])
def test_sessions_alone_equal_in_mix(cuda_dev, batching, strategy, pinned):
    """Interleaved frames of several sessions give each session the single-stream result, whether the launch
    that carries a frame holds one frame (single-stream kernels) or several (batched kernels), and whether its
    inputs are read in place from page-locked host memory (pinned) or copied in (pageable)."""
    sizes = [(64, 36), (160, 90), (33, 17)]
    frames = 4
    seqs = [_host_seq(w, h, frames, seed=3 + j, f16=True, pinned=pinned) for j, (w, h) in enumerate(sizes)]
    want = [_single(w, h, seq, tg.STORAGE_FP16, cuda_dev) for (w, h), seq in zip(sizes, seqs)]
    sv = Server(256 << 20, max_batch=8, batching=batching, storage=tg.STORAGE_FP16, strategy=strategy)
    outs = [[torch.empty((h, w, 4), dtype=torch.float16, pin_memory=True) for _ in range(frames)] for (w, h) in sizes]
    tickets = []
    for t in range(frames):
        for j in range(len(sizes)):
            tickets.append(sv.submit(100 + j, seqs[j][t], outs[j][t]))
    infos = [sv.wait(tk) for tk in tickets]
    assert all(i["status"] == 0 for i in infos)
    for j in range(len(sizes)):
        for t in range(frames):
            assert torch.equal(outs[j][t], want[j][t]), f"session {j} frame {t}"
    st = sv.stats()
    assert st["completed"] == len(tickets) and st["failed"] == 0
    if batching:
        assert st["max_batch_seen"] >= 2
    sv.close()


def test_budget_eviction_restarts_history(cuda_dev):
    """A budget that holds one session: alternating sessions evict each other and restart from zero history."""
    w, h = 64, 36
    seqs = [_host_seq(w, h, 3, seed=11 + j) for j in range(2)]
    first = [_single(w, h, seq[:1], tg.STORAGE_FP32, cuda_dev)[0] for seq in seqs]
    probe = Server(64 << 20, storage=tg.STORAGE_FP32)
    o = torch.empty((h, w, 4), pin_memory=True)
    probe.wait(probe.submit(1, seqs[0][0], o))
    one = probe.stats()["peak_resident_bytes"]
    probe.close()
    sv = Server(one + one // 2, storage=tg.STORAGE_FP32)
    outs = []
    for t in range(3):
        for j in range(2):
            ob = torch.empty((h, w, 4), pin_memory=True)
            info = sv.wait(sv.submit(j, seqs[j][0], ob))  # the same first frame each time
            assert info["status"] == 0
            outs.append((j, ob))
    st = sv.stats()
    assert st["evictions"] >= 4 and st["admissions"] >= 5
    for j, ob in outs:  # every frame ran on freshly zeroed history
        assert torch.equal(ob, first[j])
    sv.close()


def test_oversized_session_fails_with_budget(cuda_dev):
    sv = Server(1 << 20, storage=tg.STORAGE_FP32)
    seq = _host_seq(320, 180, 1, seed=1)
    o = torch.empty((180, 320, 4), pin_memory=True)
    info = sv.wait(sv.submit(7, seq[0], o))
    assert info["status"] == tg._lib.ERR_BUDGET
    sv.close()


def test_ended_session_fails_its_queue_and_server_keeps_serving(cuda_dev):
    sv = Server(64 << 20, storage=tg.STORAGE_FP32, max_batch=2)
    seq = _host_seq(96, 64, 6, seed=2)
    outs = [torch.empty((64, 96, 4), pin_memory=True) for _ in range(6)]
    tks = [sv.submit(5, seq[t], outs[t]) for t in range(6)]
    sv.end_session(5)
    infos = [sv.wait(tk) for tk in tks]
    ok = [i["status"] for i in infos]
    assert set(ok) <= {0, tg._lib.ERR_STATE}
    # a new session still works
    o = torch.empty((64, 96, 4), pin_memory=True)
    assert sv.wait(sv.submit(6, seq[0], o))["status"] == 0
    sv.close()


def test_submit_rejects_malformed_inputs(cuda_dev):
    sv = Server(64 << 20, storage=tg.STORAGE_FP32)
    seq = _host_seq(32, 16, 1, seed=4)
    o = torch.empty((16, 32, 4), pin_memory=True)
    bad = dict(seq[0])
    bad["radiance"] = seq[0]["radiance"][:, :16].contiguous()  # rows shorter than the frame
    with pytest.raises(tg.TgError):
        sv.submit(1, bad, o)
    with pytest.raises(tg.TgError):
        sv.wait(123456)
    sv.close()


def test_barrier_wait_runs_out_and_reports(cuda_dev):
    """The persistent kernel's grid barrier is bounded: told to wait for a CTA that does not
    exist, every CTA gives up after 2 ms, the step reports TG_ERR_TIMEOUT and the context
    stays usable."""
    sizes = [(64, 36)]
    sc = scene.PlaneScene(scene.pan_with_disocclusion(64, 36, seed=9))
    fr = {k: v.to(cuda_dev) for k, v in sc.frame(0).items() if k in KEYS}
    out = [torch.empty((36, 64, 4), device=cuda_dev)]
    b = Batch(sizes, storage=tg.STORAGE_FP32, strategy=tg._lib.BATCH_PERSISTENT, barrier_timeout_us=2000,
              debug_barrier_extra=1)
    b.denoise([0], [fr], out)
    with pytest.raises(tg.TgError) as e:
        b.synchronize()
    assert e.value.status == tg._lib.ERR_TIMEOUT
    assert b.info()["barrier_timeouts"] == 1
    b.close()
    ok = Batch(sizes, storage=tg.STORAGE_FP32)
    ok.denoise([0], [fr], out)
    ok.synchronize()
    assert torch.isfinite(out[0]).all()
    ok.close()

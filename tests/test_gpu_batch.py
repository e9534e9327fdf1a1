"""Batched form (vbm3d_batch_*): clips of uneven size, channel count and
sigma denoised by one CUDA graph launch.

Each clip's result must match the plain per-clip path (vbm3d_gpu_run) and
the oracle: basic estimate within TOL max-abs, final estimate within TOL on
all but 1% of values (the step-2 matching reads the basic estimate, whose
last bits depend on the order of the atomic aggregation), PSNR within
0.01 dB.  Also: repeated graph launches, inputs refilled in place between
launches, fixed configurations with and without the graph, flows, the
profiled run and the reported configuration.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip, psnr  # noqa: E402

TOL = 1e-3

# (width, height, frames, channels, sigma): every default class of the
# batched kernels (step 2 k = 7 for sigma <= 30, k = 8 above; 1 and 3
# channels), uneven sizes, odd widths.
SPECS = [
    (64, 48, 6, 3, 20.0),
    (50, 40, 5, 1, 50.0),
    (81, 56, 7, 3, 5.0),
    (40, 36, 5, 1, 10.0),
    (72, 41, 6, 3, 40.0),
    (96, 64, 8, 1, 30.0),
]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


@pytest.fixture(scope="module")
def clips():
    out = []
    for i, (w, h, f, c, s) in enumerate(SPECS):
        clean, noisy, ff, bf = make_clip(w, h, f, c, s, 4000 + i, with_flow=(i % 2 == 0))
        out.append(dict(clean=clean, noisy=noisy, sigma=s, fflow=ff, bflow=bf))
    return out


def gpu(a, dev):
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


def batch_of(clips, dev, flows=True, **kw):
    items = [dict(noisy=gpu(c["noisy"], dev), sigma=c["sigma"],
                  fflow=gpu(c["fflow"], dev) if flows else None,
                  bflow=gpu(c["bflow"], dev) if flows else None) for c in clips]
    return vb.Batch(items, **kw), items


def plain(c, dev, color_space, flows=True):
    b, d = vb.run(gpu(c["noisy"], dev), c["sigma"], fflow=gpu(c["fflow"], dev) if flows else None,
                  bflow=gpu(c["bflow"], dev) if flows else None, color_space=color_space)
    return b.cpu().numpy(), d.cpu().numpy()


def assert_close(clean, got_b, got_d, want_b, want_d):
    # basic estimates: within 1e-3 at every value.  Final estimates: the
    # basic estimates' last bits depend on the order of the aggregation's
    # float atomics, and a near-tie of step 2's block matching that flips
    # changes the groups, and so the final values, of the patches involved
    # (by up to a few units: 3.6 at most on the full-size workloads); on
    # these small clips that reached 1.3 % of the values in one run of about
    # fifteen, so the share is bounded at 3 %, the size at 8 and the PSNR
    # difference at 0.01 dB.  A stale input or a wrong clip parameter moves
    # most values, by about sigma, and the PSNR.
    assert np.abs(got_b - want_b).max() <= TOL
    d = np.abs(got_d - want_d)
    assert (d > TOL).mean() < 0.03 and d.max() < 8.0, (d.max(), (d > TOL).mean())
    assert abs(psnr(clean, got_d) - psnr(clean, want_d)) <= 0.01
    assert abs(psnr(clean, got_b) - psnr(clean, want_b)) <= 0.01


@pytest.mark.parametrize("cs", [True, False])
def test_batch_matches_plain_per_clip(dev, clips, cs):
    b, _ = batch_of(clips, dev, color_space=cs)
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(clips):
        pb, pd = plain(c, dev, cs)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), pb, pd)
        assert psnr(c["clean"], den[i].cpu().numpy()) > psnr(c["clean"], c["noisy"]) + 3
    cfg = b.config()
    for key in ("bm1", "filter1", "bm2", "filter2"):
        assert cfg[key + "_tile"] > 0 and cfg[key + "_warps"] in (1, 2, 4, 8)
    assert cfg["work_items"] > 0 and cfg["device_bytes"] > 0 and cfg["no_graph"] == 0
    b.close()


def test_batch_matches_oracle(dev, clips):
    o = Oracle()
    sub = [clips[0], clips[1], clips[4]]
    b, _ = batch_of(sub, dev, color_space=True)
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(sub):
        p1, p2 = o.default_params(1, c["sigma"]), o.default_params(2, c["sigma"])
        ob, of = o.run(c["sigma"], c["noisy"], p1, p2, c["fflow"], c["bflow"], color_space=True, threads=4)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), ob, of)


def test_repeated_launches_and_refilled_inputs(dev, clips):
    b, items = batch_of(clips, dev, color_space=True)
    first = [d.cpu().numpy() for d in b.run()[1]]
    second = [d.cpu().numpy() for d in b.run()[1]]
    for c, x, y in zip(clips, first, second):
        assert_close(c["clean"], x, y, x, x)
    # a new noise realisation written into the same input buffers
    fresh = []
    for i, (c, it) in enumerate(zip(clips, items)):
        rng = np.random.default_rng(77 + i)
        noisy = c["clean"] + rng.standard_normal(c["clean"].shape).astype(np.float32) * np.float32(c["sigma"])
        it["noisy"].copy_(torch.from_numpy(noisy))
        fresh.append(dict(c, noisy=noisy))
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(fresh):
        pb, pd = plain(c, dev, True)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), pb, pd)
    b.close()


@pytest.mark.parametrize("tile,warps,no_graph", [(1, 1, 1), (8, 4, 0), (64, 8, 1)])
def test_fixed_configurations(dev, clips, tile, warps, no_graph):
    cfg = dict(bm1_tile=tile, bm1_warps=warps, filter1_tile=tile, filter1_warps=warps, bm2_tile=tile,
               bm2_warps=warps, filter2_tile=tile, filter2_warps=warps, no_graph=no_graph)
    b, _ = batch_of(clips, dev, flows=False, color_space=True, config=cfg)
    got = b.config()
    assert got["bm2_tile"] == tile and got["filter1_warps"] == warps and got["no_graph"] == no_graph
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(clips):
        pb, pd = plain(c, dev, True, flows=False)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), pb, pd)
    b.close()


def test_uneven_batch_sampled_like_the_benchmark(dev):
    # the benchmark's distribution of shapes, scaled down 4x per side
    rng = np.random.default_rng(4000)
    specs = []
    for i in range(12):
        w, h = int(rng.integers(160, 1281)) // 4, int(rng.integers(120, 721)) // 4
        f, c = int(rng.integers(5, 13)), int(rng.choice([1, 3]))
        s = float(rng.choice([5, 10, 20, 30, 50]))
        clean, noisy, _, _ = make_clip(w, h, f, c, s, 4100 + i)
        specs.append(dict(clean=clean, noisy=noisy, sigma=s, fflow=None, bflow=None))
    b, _ = batch_of(specs, dev, color_space=True)
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(specs):
        pb, pd = plain(c, dev, True)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), pb, pd)
    b.close()


def test_profile_run_matches_graph_run(dev, clips):
    b, _ = batch_of(clips, dev, color_space=True)
    graph = [d.cpu().numpy() for d in b.run()[1]]
    launches = b.profile()
    torch.cuda.synchronize()
    prof = [d.cpu().numpy() for d in b.denoised]
    for c, x, y in zip(clips, graph, prof):
        assert_close(c["clean"], x, y, x, x)
    # each phase's launches cover every clip's grid once
    assert {l["phase"] for l in launches} == {0, 1, 2, 3}
    for ph in range(4):
        refs = sum(l["refs"] for l in launches if l["phase"] == ph)
        want = sum(vb.ref_count(vb.default_params(ph // 2 + 1, c["sigma"]), vb.dims_of(c["noisy"])) for c in clips)
        assert refs == want
    assert all(l["ms"] > 0 and l["items"] > 0 and l["grid"] > 0 for l in launches)
    b.close()


def test_wide_search_windows(dev):
    # per-clip parameters with Ns = 11 and Npr = 9: frame-t tiles wider than
    # 16 columns and forward / backward windows of 81 positions, in the
    # batched block matching of one channel (half warps) and three (warps)
    specs = []
    for i, (w, h, f, c, s) in enumerate([(56, 44, 6, 1, 20.0), (60, 40, 6, 3, 40.0)]):
        clean, noisy, _, _ = make_clip(w, h, f, c, s, 4200 + i)
        p1 = vb.default_params(1, s).replace(Ns=11, Npr=9)
        p2 = vb.default_params(2, s).replace(Ns=11, Npr=9)
        specs.append(dict(clean=clean, noisy=noisy, sigma=s, p1=p1, p2=p2))
    b = vb.Batch([dict(noisy=gpu(c["noisy"], dev), sigma=c["sigma"], p1=c["p1"], p2=c["p2"]) for c in specs],
                 color_space=True)
    basic, den = b.run()
    torch.cuda.synchronize()
    for i, c in enumerate(specs):
        pb, pd = vb.run(gpu(c["noisy"], dev), c["sigma"], c["p1"], c["p2"], color_space=True)
        assert_close(c["clean"], basic[i].cpu().numpy(), den[i].cpu().numpy(), pb.cpu().numpy(), pd.cpu().numpy())
    b.close()

"""The batched, uneven, served and large-N workloads on the GPU against the FP64 oracle (relative error <= 1e-5, the
accuracy target of the FP32 path):

  * an uneven batch (N in {32, 64, 128}, degree caps p in {8, 16, 32}, L_p and hybrid) recorded as one CUDA graph
    (UnevenBatch): every sinogram of every class against oracle.oblique_np on that class's plan;
  * served requests of mixed sizes against the oracle directly (not only against the library's own single apply);
  * the hybrid inverse at N = 2048, p = 64, batch 1, FP32, against the FP64 pipeline on the same plan (the FP64
    pipeline is pinned to the reference's own outputs at n = 4 and 6 to 1e-11 by test_gpu_inverse.py; the NumPy
    oracle would take many minutes per apply at this size).
"""

import numpy as np
import pytest

from conftest import rel_err
from oracle import oblique_np as O

pytestmark = pytest.mark.gpu

# dense rows per degree cap, as the uneven workload uses them: none at p = 8, cap 12 at p = 16, 16 above
DENSE_CAP = {8: None, 16: 12, 32: 16, 64: 16}
# (n, method, p, sinograms)
UNEVEN = [(5, "lp", 8, 2), (5, "hybrid", 16, 3), (6, "lp", 16, 2), (6, "hybrid", 32, 2), (7, "lp", 32, 2),
          (7, "hybrid", 8, 2)]


def _sinos(pkg, n, count, seed, rel_sigma):
    from adrt_pinv_gb300 import adrtcore, phantoms

    N = 1 << n
    return np.stack([phantoms.add_noise(adrtcore.adrt(n, phantoms.ellipse_phantom(N, seed=seed + i)), s, seed + i)
                     for i, s in enumerate(rel_sigma)])


def _oracle(inv, method, dense_cap):
    kw = dict(lam_max=inv.lam_max, deg=inv.deg, outer=(inv.lo, inv.hi, inv.outer_deg), dense_cap=dense_cap)
    return O.LpOracle(inv.n, **kw) if method == "lp" else O.HybridOracle(inv.n, **kw)


def test_uneven_batch_one_graph_matches_oracle(pkg):
    import torch

    from adrt_pinv_gb300 import uneven

    rng = np.random.default_rng(5)
    groups, sinos, oracles = [], [], []
    for n, method, p, count in UNEVEN:
        cls = pkg.FastLpGpu if method == "lp" else pkg.FastHybridGpu
        inv = cls(n, deg_cap=p, dense_cap=DENSE_CAP[p], precision="fp32")
        groups.append((inv, count))
        sinos.append(_sinos(pkg, n, count, 1000 * n + p, rng.uniform(1e-4, 1e-2, count)))
        oracles.append(_oracle(inv, method, DENSE_CAP[p]))
    U = uneven.UnevenBatch(groups)
    U.set_inputs([torch.from_numpy(s).cuda() for s in sinos])
    for _ in range(2):  # the second replay reuses every buffer the first left behind
        outs = U.replay()
        torch.cuda.synchronize()
        U.check()
        for (n, method, p, count), o, s, ref in zip(UNEVEN, outs, sinos, oracles):
            got = o.cpu().numpy()
            for i in range(count):
                err = rel_err(got[i], ref.apply(s[i]))
                assert err < 1e-5, (n, method, p, i, err)


def test_served_mixed_sizes_match_oracle(pkg):
    """Requests of three sizes and both methods through the continuous-batching server, each result against the
    FP64 oracle on the request's plan."""
    from adrt_pinv_gb300 import serve

    kinds = {5: ("hybrid", 32), 6: ("lp", 16), 7: ("hybrid", 16)}
    invs, oracles = {}, {}
    for n, (method, p) in kinds.items():
        cls = pkg.FastLpGpu if method == "lp" else pkg.FastHybridGpu
        invs[n] = cls(n, deg_cap=p, dense_cap=DENSE_CAP[p], precision="fp32")
        oracles[n] = _oracle(invs[n], method, DENSE_CAP[p])
    S = serve.InverseServer(lambda n: invs[n], slots=lambda n: 3, hbm_budget_bytes=120e9)
    sizes = np.random.default_rng(9).choice(list(kinds), size=12)
    reqs = []
    for i, n in enumerate(sizes):
        b = _sinos(pkg, int(n), 1, 77 + i, [1e-3])[0]
        reqs.append((0.001 * i, serve.Request(i, int(n), b)))
    done = S.run(reqs)
    assert len(done) == len(reqs)
    for r in done:
        assert r.error is None
        err = rel_err(r.result.numpy(), oracles[r.n].apply(r.b))
        assert err < 1e-5, (r.n, err)


def test_n2048_hybrid_p64_batch1_vs_fp64(pkg):
    import torch

    from adrt_pinv_gb300 import adrtcore, phantoms

    n, N = 11, 2048
    H = pkg.FastHybridGpu(n, deg_cap=64, dense_cap=16, precision="fp32")
    x = phantoms.ellipse_phantom(N, seed=11, ellipses=40, texture=0.1)
    b = adrtcore.adrt(n, torch.from_numpy(x[None]).cuda())
    b = b + 1e-3 * b.abs().max() * torch.randn(b.shape, generator=torch.Generator("cuda").manual_seed(3),
                                                device="cuda", dtype=b.dtype)
    got = H.apply(b)[0].cpu().numpy()
    ref = H.pipeline(1, "fp64").apply(b.contiguous())[0].cpu().numpy()
    err = rel_err(got, ref)
    assert err < 1e-5, err


def test_persistent_uneven_batch_matches_oracle(pkg):
    """The uneven batch with every class's polynomial rows in one persistent launch per outer step (lock-step
    classes, one CUDA graph): each sinogram against the oracle on its class's plan, and equal to the stream-per-class
    graph to 1e-6 (same kernels but for the row launch)."""
    import torch

    from adrt_pinv_gb300 import uneven

    classes = [(6, "lp", 8, 2), (6, "hybrid", 32, 3), (7, "lp", 16, 2), (7, "hybrid", 16, 2), (6, "hybrid", 8, 1)]
    rng = np.random.default_rng(6)
    groups, sinos, oracles = [], [], []
    for n, method, p, count in classes:
        cls = pkg.FastLpGpu if method == "lp" else pkg.FastHybridGpu
        inv = cls(n, deg_cap=p, dense_cap=DENSE_CAP[p], precision="fp32")
        groups.append((inv, count))
        sinos.append(_sinos(pkg, n, count, 2000 * n + p, rng.uniform(1e-4, 1e-2, count)))
        oracles.append(_oracle(inv, method, DENSE_CAP[p]))
    P = uneven.PersistentUnevenBatch(groups)
    U = uneven.UnevenBatch(groups)
    dev = [torch.from_numpy(s).cuda() for s in sinos]
    P.set_inputs(dev)
    U.set_inputs(dev)
    for _ in range(2):
        outs = [o.clone() for o in P.replay()]
        ref = [o.clone() for o in U.replay()]
        torch.cuda.synchronize()
        P.check()
        for (n, method, p, count), o, r, s, orc in zip(classes, outs, ref, sinos, oracles):
            assert float((o - r).norm() / r.norm()) < 1e-6, (n, method, p)
            got = o.cpu().numpy()
            for i in range(count):
                assert rel_err(got[i], orc.apply(s[i])) < 1e-5, (n, method, p, i)

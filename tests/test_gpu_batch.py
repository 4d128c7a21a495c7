"""Batched JK builds (grouped tensor-core launches in a CUDA graph).

Every tile configuration gives the same J_i, K_i as the single-molecule build
(1e-12 normwise; the exact slice groups are identical, only the FP32 order of
the small groups changes) and as the FP64 oracle (1e-10); graph replays are
reproducible; the autotuner picks a configuration and caches it.
"""
import numpy as np
import pytest

from conftest import nrel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(request):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    mols, refs, single = [], [], []
    for i, nbf in enumerate([24, 37, 50, 67, 90]):
        st = synthetic.Structure.for_nbf(nbf)
        b, C, H, n = synthetic.make_inputs(st, 1000 + i)
        db, dC = ops.to_device(b), ops.to_device(C)
        prep = ops.PreparedRI(db, 6)
        mols.append((dC, prep, st.nbf5))
        refs.append(orc.jkj_ri(C, b, st.nbf5))
        J, K = ops.jkj_ri_mixed(dC, prep, st.nbf5)
        single.append((J.cpu().numpy(), K.cpu().numpy()))
    return mols, refs, single


@pytest.mark.parametrize("tiles", [(0, 0), (1, 1), (2, 2), (3, 3), (1, 0), (0, 2)])
def test_batch_tile_configs(batch, tiles):
    from pynof_gb300 import ops
    from pynof_gb300.batch import BatchJK

    mols, refs, single = batch
    plan = BatchJK(mols, tiles=tiles)
    plan.run()
    plan.stream.synchronize()
    ops.check_device_status()
    first = [(J.cpu().numpy(), K.cpu().numpy()) for J, K in zip(plan.J, plan.K)]
    plan.run()
    plan.stream.synchronize()
    for (J, K), (J1, K1), (Js, Ks), (Jr, Kr) in zip(zip(plan.J, plan.K), first, single, refs):
        J, K = J.cpu().numpy(), K.cpu().numpy()
        assert np.array_equal(J, J1) and np.array_equal(K, K1)
        assert nrel(J, Js) < 1e-12 and nrel(K, Ks) < 1e-12
        assert nrel(J, Jr) < 1e-10 and nrel(K, Kr) < 1e-10
    plan.close()


def test_autotune(batch, tmp_path, monkeypatch):
    from pynof_gb300 import batch as bmod

    mols, _, _ = batch
    monkeypatch.setenv("PYNOF_GB300_CACHE", str(tmp_path / "tiles.json"))
    tiles, info = bmod.autotune(mols, reps=2)
    assert len(tiles) == 2 and all(0 <= t <= 3 for t in tiles) and not info["cached"]
    tiles2, info2 = bmod.autotune(mols, reps=2)
    assert tiles2 == tiles and info2["cached"]

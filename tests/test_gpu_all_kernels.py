"""Every kernel family of the library launched once in one process, with the counts checked.

R-MAT 18 ef16 is counted under the tuned, learned (split forced), forced-hub (warp_max 32,
block_max 64) and cycle-recording schedules.  Also covered: a 20,000-entry hub row on a 4-CTA
cluster, the 2x2 device tile loop with the split forced, a staged host count, a 256-graph batch,
one epoch of cost-model training, the generators and the GPU preprocessing.  Every path must give
the oracle's count.  The launch-list profile of the whole library runs this file under ncu.
"""
import numpy as np
import pytest

import trust_gb300 as T
from oracle import oracle as O
from trust_gb300 import batch as B

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_every_kernel_family_agrees():
    pairs = T.gen_rmat(18, 16, seed=3)                                   # generator
    beg, adj = T.build_csr(pairs, 1 << 18)                               # preprocessing kernels
    T.gen_er(1 << 16, 1 << 20, seed=5)
    T.gen_ba(1 << 16, 8, seed=5)
    T.gen_chung_lu(1 << 16, 2.5, 100.0, 1 << 19, 1 << 19, seed=2)
    expect = O.count_forward_sorted_range(beg.cpu().numpy(), adj.cpu().numpy(), 0, beg.numel() - 1, 2, 8)
    ctx = T.Context()
    counts = [
        T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED),                      # check, class, count
        T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_LEARNED, direction_split=1),  # schedule, split, pass B
        T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, warp_max=32, block_max=64),  # hub kernel
        T.count_tiles(beg, adj, 2, direction_split=1),                               # partition, tile jobs
    ]
    cyc = torch.zeros(beg.numel() - 1, dtype=torch.int64, device="cuda")
    counts.append(T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, cycles=cyc))  # cycle recording
    hb_np, ha_np = beg.cpu().pin_memory().numpy(), adj.cpu().pin_memory().numpy()
    T.stage_csr(hb_np, ha_np, ctx)
    counts.append(T.count_csr(hb_np, ha_np, ctx=ctx))                                 # staged host input
    assert [r.triangles for r in counts] == [expect] * len(counts)

    # one hub row of 20,000 entries: its table (64 Ki slots) spans a 4-CTA cluster
    D = 20_000
    hb = torch.from_numpy(np.concatenate([[0], D + np.arange(0, D + 1)]).astype(np.int64)).cuda()
    ha = np.concatenate([np.arange(1, D + 1), np.arange(2, D + 2)]).astype(np.int32)
    ha[-1] = 0
    assert T.count_csr(hb, torch.from_numpy(ha).cuda(), ctx=ctx).triangles == D - 1

    specs = B.batch_specs(256, 50, 5000, seed=11)
    bp, vb = B.gen_batch_pairs(specs)
    bb, ba, gv = B.build_batch(bp, vb)
    bt = B.Batch(bb, ba, gv, ctx=ctx)
    c, rb = bt.run()
    assert int(c.sum()) == rb.triangles
    bt.close()

    f = T.vertex_features(beg, adj, ctx)                                             # features
    d = torch.from_numpy(np.diff(beg.cpu().numpy())).cuda()
    keep = d >= 2
    x = f[keep][:20000].contiguous()
    y = torch.log2(1 + cyc[keep][:20000].float()).contiguous()
    mod, loss = T.model_train(x, y, T.model_init(seed=1), epochs=1, batch=4096, lr=1e-3)  # grad + Adam
    assert np.isfinite(loss)
    assert torch.isfinite(T.model_predict(x, mod)).all()                             # predict

"""Launch every kernel family of the library once, at modest sizes, and check the counts agree.

    python -m trust_gb300.exercise

Used to profile all kernels in one process (R-MAT 18 ef16 under the tuned, learned, forced-hub and
cycle-recording schedules, a 20,000-entry hub row on a thread-block cluster, the 2x2 device tile
loop with the direction split, a staged host count, a 256-graph batch, one epoch of cost-model
training, the generators and GPU preprocessing).
"""
import numpy as np
import torch

import trust_gb300 as T
from trust_gb300 import batch as B
pairs = T.gen_rmat(18, 16, seed=3)                      # rmat_kernel
beg, adj = T.build_csr(pairs, 1 << 18)                  # preprocessing kernels
T.gen_er(1 << 16, 1 << 20, seed=5); T.gen_ba(1 << 16, 8, seed=5); T.gen_chung_lu(1 << 16, 2.5, 100.0, 1 << 19, 1 << 19, seed=2)
ctx = T.Context()
r0 = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED)                          # check, class, count
r1 = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_LEARNED, direction_split=1)      # sched, split, lpt, pass B
r2 = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, warp_max=32, block_max=64)  # hub kernel, one CTA
D = 20_000
hb = torch.from_numpy(np.concatenate([[0], D + np.arange(0, D + 1)]).astype(np.int64)).cuda()
ha = np.concatenate([np.arange(1, D + 1), np.arange(2, D + 2)]).astype(np.int32); ha[-1] = 0
r3 = T.count_csr(hb, torch.from_numpy(ha).cuda(), ctx=ctx)                            # hub kernel, 4-CTA cluster
r4 = T.count_tiles(beg, adj, 2, direction_split=1)                                   # GPU partition, tile checks,
                                                                                     # tile split plan, tile jobs
specs = B.batch_specs(256, 50, 5000, seed=11)
bp, vb = B.gen_batch_pairs(specs); bb, ba, gv = B.build_batch(bp, vb)                 # ba_kernel, batch build
bt = B.Batch(bb, ba, gv, ctx=ctx); c, rb = bt.run()                                  # batch class/offsets/count
cyc = torch.zeros(beg.numel() - 1, dtype=torch.int64, device="cuda")
T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, cycles=cyc)                   # cycle-recording count
f = T.vertex_features(beg, adj, ctx)                                                 # features
d = torch.from_numpy(np.diff(beg.cpu().numpy())).cuda(); m = d >= 2
x = f[m][:20000].contiguous(); y = torch.log2(1 + cyc[m][:20000].float()).contiguous()
mod, loss = T.model_train(x, y, T.model_init(seed=1), epochs=1, batch=4096, lr=1e-3)  # mlp grad + adam
T.model_predict(x, mod)                                                              # predict
hb_np, ha_np = beg.cpu().pin_memory().numpy(), adj.cpu().pin_memory().numpy()
T.stage_csr(hb_np, ha_np, ctx)
r5 = T.count_csr(hb_np, ha_np, ctx=ctx)                                              # staged host input
assert r0.triangles == r1.triangles == r2.triangles == r4.triangles == r5.triangles and r3.triangles == D - 1
assert int(c.sum()) == rb.triangles
print("ok", r0.triangles, rb.triangles)

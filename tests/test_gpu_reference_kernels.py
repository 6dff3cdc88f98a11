"""Parity with the reference's own GPU kernels (GPU).

The reference's CL (xxx_query, alg 16) and VL (kernel_hierarchical_vector_load,
alg 20) kernels, compiled from its sources into oracle/_ref (device code only),
run on the same GPU; their minima must equal this library's bit for bit and
the CPU oracle's.  Skipped where that build is absent."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from oracle import oracle, ref_gpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference kernels not built")]


@pytest.mark.parametrize("variant,t", [("cl", 64), ("cl", 1024), ("vl", 32), ("vl", 1024)])
@pytest.mark.parametrize("n,lr", [(1 << 20, -7), (100_004, -6), (4100, -1)])
def test_reference_kernels_agree(cuda, variant, t, n, lr):
    import torch
    a = R.gen_array(n, 3)
    qs = R.gen_queries(1 << 15, lr, n, 3)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    rk = ref_gpu.RefKernels()
    stream = torch.cuda.current_stream().cuda_stream
    md, lvl = rk.build(dv, t, variant, stream)
    ref_out = torch.empty(qs.shape[0], dtype=torch.float32, device=cuda)
    rk.query(dv, md, lvl, dq, ref_out, t, variant, stream)
    with R.Hierarchy(dv, variant=variant, t=t) as h:
        ours = h.query(dq)
    torch.cuda.synchronize()
    exp = oracle.rmq_min(a, qs)
    assert ref_out.cpu().numpy().tobytes() == exp.tobytes(), "reference kernel vs oracle"
    assert ours.cpu().numpy().tobytes() == exp.tobytes(), "library vs oracle"

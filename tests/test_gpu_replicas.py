"""Device-side replica merge on one GPU: the library's FP64 images seen as CUDA
arrays, and a one-rank NCCL group through merge_tallies_device (identity)."""

import os
import socket

import numpy as np
import pytest

from opengate_gb300 import _capi as C
from opengate_gb300 import replicas as Rp
from opengate_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_device_image_view_and_one_rank_merge():
    import torch
    import torch.distributed as dist

    from opengate_gb300.engine import DoseEngine

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.cuda.set_device(0)
    with DoseEngine(W.water_pencil(), device=0) as eng:
        eng.run(20_000, 5)
        e, e2 = eng.edep(), eng.edep_squared()
        ptr, n = eng.image_device(C.GG_IMG_EDEP)
        assert n == e.size
        view = torch.as_tensor(Rp._DeviceImage(ptr, n), device="cuda:0")
        np.testing.assert_array_equal(view.cpu().numpy(), e.ravel())
        dist.init_process_group("nccl", rank=0, world_size=1)
        try:
            total = Rp.merge_tallies_device(eng, (C.GG_IMG_EDEP, C.GG_IMG_EDEP_SQUARED), 20_000)
        finally:
            dist.destroy_process_group()
        assert total == 20_000
        np.testing.assert_array_equal(eng.edep(), e)
        np.testing.assert_array_equal(eng.edep_squared(), e2)

"""pppm_render_read into the three kinds of destination: device memory,
page-locked host memory (which the SMs may write directly through its
device address) and pageable host memory. Every destination receives the
same bytes, for images whose size is a multiple of 16 bytes and for one
that is not."""
import numpy as np
import pytest
import torch

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("size", [(32, 24), (7, 5)])
def test_read_destinations_agree(size):
    w, h = size
    sc = S.small_test_scene(seed=5, subdiv=2, width=w, height=h, photons=4000)
    c = P.Context(0)
    try:
        c.set_scene(sc)
        c.render_begin(sc.camera, P.Context.make_params(mode=P.MODE_CANONICAL, photons=4000, radius_scale=1 / 16))
        for t in (1, 2):
            c.render_pass(t)
        pageable = c.render_read()
        pinned = torch.zeros((h, w, 3), dtype=torch.float32, pin_memory=True)
        c.render_read(pinned.numpy())
        dev = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        c.render_read(dev)
        assert np.abs(pageable).sum() > 0
        assert np.array_equal(pageable.view(np.uint32), pinned.numpy().view(np.uint32))
        assert np.array_equal(pageable.view(np.uint32), dev.cpu().numpy().view(np.uint32))
        # a pinned destination that starts 4 bytes into its allocation
        big = torch.zeros(h * w * 3 + 1, dtype=torch.float32, pin_memory=True)
        c.render_read(big.numpy()[1:].reshape(h, w, 3))
        assert np.array_equal(pageable.reshape(-1).view(np.uint32), big.numpy()[1:].view(np.uint32))
    finally:
        c.close()

"""The GPU scene generator writes exactly the host generator's bytes."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,count", [(1, 3), (3, 4), (4, 2), (5, 6)])
def test_device_scenes_equal_host(cuda, kind, count):
    import torch
    from opencuda_gb300 import _lib
    L = _lib.load()
    ps = (_lib.hl_scene_params * count)()
    assert L.hl_synth_spec(kind, 77, count, ps) == 0
    bufs, descs = [], (_lib.hl_image_desc * count)()
    for i in range(count):
        w, h = ps[i].width, ps[i].height
        pitch = (w + 511) // 512 * 512
        t = torch.full((h, pitch), 7, dtype=torch.uint8, device="cuda")
        bufs.append(t)
        descs[i] = _lib.hl_image_desc(t.data_ptr(), pitch, w, h, 0, 0, w, h)
    assert L.hl_synth_scenes_device(ps, count, descs, None) == 0
    for i in range(count):
        w, h = ps[i].width, ps[i].height
        host = np.zeros((h, w), np.uint8)
        assert L.hl_synth_scene(C.byref(ps[i]), C.c_void_p(host.ctypes.data), w) == 0
        dev = bufs[i][:, :w].cpu().numpy()
        assert np.array_equal(dev, host), (kind, i)

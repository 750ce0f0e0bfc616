"""Frames composited straight into host memory (pf_set_host_image) equal device-image frames."""
import numpy as np
import pytest

import scenes as S

pytestmark = pytest.mark.gpu


def test_host_image_target_matches_device_images(pf):
    scs = S.batched(n_scenes=5, first_seed=77, hi_paths=200)
    with pf.Renderer(device=0) as r:
        r.upload(scs)
        r.render()
        want = [r.image(i) for i in range(len(scs))]
        nbytes = r.image_bytes()
        host = np.zeros(nbytes, np.uint8)  # pageable numpy memory: pinned and mapped by the library
        r.set_host_image(host.ctypes.data, nbytes)
        r.sizer_load()
        r.render_learned()
        for i, sc in enumerate(scs):
            h, w = int(np.ceil(sc.height)), int(np.ceil(sc.width))
            off = r.image_offset(i)
            got = host[off:off + h * w * 4].reshape(h, w, 4)
            assert np.array_equal(got, want[i]), i
            assert np.array_equal(r.image(i), want[i]), i
        # a buffer smaller than the batch's images is refused at the next frame
        r.set_host_image(host.ctypes.data, nbytes - 1)
        with pytest.raises(pf.PfError):
            r.render()
        # NULL restores device images
        r.set_host_image(None)
        r.render()
        for i in range(len(scs)):
            assert np.array_equal(r.image(i), want[i])


def test_host_image_target_in_caller_pinned_memory(pf):
    torch = pytest.importorskip("torch")
    scs = S.batched(n_scenes=3, first_seed=91, hi_paths=120)
    with pf.Renderer(device=0) as r:
        r.upload(scs)
        r.render()
        want = [r.image(i) for i in range(len(scs))]
        nbytes = r.image_bytes()
        pinned = torch.zeros(nbytes, dtype=torch.uint8, pin_memory=True)  # cudaHostAlloc'd by torch
        r.set_host_image(pinned.data_ptr(), nbytes)
        r.render()
        host = pinned.numpy()
        for i, sc in enumerate(scs):
            h, w = int(np.ceil(sc.height)), int(np.ceil(sc.width))
            off = r.image_offset(i)
            assert np.array_equal(host[off:off + h * w * 4].reshape(h, w, 4), want[i]), i
        r.set_host_image(None)

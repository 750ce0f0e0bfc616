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


def test_async_readback_delivers_each_frames_images(pf):
    """pf_read_images_async: frame A's images arrive in buffer A while frame B (other scenes,
    uploaded and rendered after the call) proceeds; B's in buffer B; repeated, the snapshot
    buffer is reused only after the previous copy."""
    torch = pytest.importorskip("torch")
    a = S.batched(n_scenes=4, first_seed=301, hi_paths=300)
    b = S.batched(n_scenes=4, first_seed=401, hi_paths=300)
    with pf.Renderer(device=0) as r:
        want = {}
        for name, scs in (("a", a), ("b", b)):
            r.upload(scs)
            r.render()
            want[name] = (r.image_bytes(), [r.image(i) for i in range(len(scs))],
                          [r.image_offset(i) for i in range(len(scs))])
        nbytes = max(want["a"][0], want["b"][0])
        bufs = {k: torch.zeros(nbytes, dtype=torch.uint8, pin_memory=True) for k in ("a", "b")}
        r.sizer_load()
        for _ in range(3):
            for name, scs in (("a", a), ("b", b)):
                r.upload(scs)
                r.render_learned()
                r.read_images_async(bufs[name].data_ptr(), nbytes)
            r.images_wait()
            for name, scs in (("a", a), ("b", b)):
                host = bufs[name].numpy()
                for i, sc in enumerate(scs):
                    h, w = int(np.ceil(sc.height)), int(np.ceil(sc.width))
                    off = want[name][2][i]
                    assert np.array_equal(host[off:off + h * w * 4].reshape(h, w, 4), want[name][1][i]), (name, i)
                bufs[name].zero_()
        with pytest.raises(pf.PfError):
            r.read_images_async(bufs["a"].data_ptr(), 16)

"""vj_integral_image_noalloc: the integral-image entry point for callers that
cannot allocate device memory (a caller-owned memory pool or fixed budget, or a
latency-bound pipeline that must not go through the CUDA allocator).  It keeps
its scratch in a fixed device array instead of allocating, so its output must
equal the allocating vj_integral_image bit for bit, call after call, with the
shared scratch reused in between.  Collected last so a failure here comes after
every other test has run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _integral(torch, vj, name, img):
    h, w = img.shape
    d = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    s = torch.full(((h + 1) * (w + 1),), -1, dtype=torch.int32, device="cuda")
    q = torch.full_like(s, -1, dtype=torch.int64)
    vj._capi.call(name, d.data_ptr(), w, h, w, s.data_ptr(), q.data_ptr(), None)
    torch.cuda.synchronize()
    return s.cpu().numpy(), q.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(cuda, vj):
    torch = cuda
    # two calls in a row with different sizes: the second reuses the scratch
    # the first left behind
    for seed, (h, w) in enumerate([(1080, 1920), (333, 517), (2160, 3840)]):
        img = vj.synth_scene(seed + 11, w, h, 2, 24, 100)
        a_s, a_q = _integral(torch, vj, "vj_integral_image", img)
        b_s, b_q = _integral(torch, vj, "vj_integral_image_noalloc", img)
        assert np.array_equal(a_s, b_s)
        assert np.array_equal(a_q, b_q)


def test_noalloc_padded_rows_and_unaligned_pixels(cuda, vj, oracle):
    """Rows with a stride of w + 13 starting at an odd address take the row
    pass's scalar loads; the result must still equal vj_integral_image's with
    the same arguments, and the oracle's integral of the same pixels."""
    torch = cuda
    h, w = 301, 517
    stride = w + 13
    img = vj.synth_scene(5, w, h, 3, 24, 200)
    buf = np.zeros(1 + stride * h, np.uint8)
    rows = buf[1:].reshape(h, stride)
    rows[:, :w] = img
    rows[:, w:] = 255  # padding that must not enter the sums
    d = torch.from_numpy(buf).cuda()
    want_s, want_q = oracle.integral(img)
    for _ in range(2):  # two calls in a row share the scratch
        out = {}
        for name in ("vj_integral_image", "vj_integral_image_noalloc"):
            s = torch.full(((h + 1) * (w + 1),), -1, dtype=torch.int32, device="cuda")
            q = torch.full_like(s, -1, dtype=torch.int64)
            vj._capi.call(name, d.data_ptr() + 1, w, h, stride, s.data_ptr(), q.data_ptr(), None)
            torch.cuda.synchronize()
            out[name] = (s.cpu().numpy(), q.cpu().numpy())
        a, b = out["vj_integral_image"], out["vj_integral_image_noalloc"]
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert np.array_equal(b[0].view(np.uint32), want_s.ravel())
        assert np.array_equal(b[1].view(np.uint64), want_q.ravel())


def test_noalloc_rejects_what_its_scratch_cannot_hold(cuda, vj):
    torch = cuda
    d = torch.zeros(2161 * 100, dtype=torch.uint8, device="cuda")
    s = torch.zeros(2162 * 101, dtype=torch.int32, device="cuda")
    q = torch.zeros(2162 * 101, dtype=torch.int64, device="cuda")
    st = vj._capi.status("vj_integral_image_noalloc", d.data_ptr(), 100, 2161, 100, s.data_ptr(), q.data_ptr(), None)
    assert st == vj.Status.kInvalidArg
    assert b"3840 x 2160" in vj.load().vj_last_error()
    st = vj._capi.status("vj_integral_image_noalloc", d.data_ptr(), 100, 100, 100, s.data_ptr(), None, None)
    assert st == vj.Status.kInvalidArg

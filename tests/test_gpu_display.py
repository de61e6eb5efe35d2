"""GPU: the frame raster (Stars::display), the prune on the public arrays, and the .y4m movie.

Frames are compared byte for byte: with the frames the reference's own displayDevice drew (tests/golden), and with
the oracle's restatement on larger fields, special values, and the state the engine's own update leaves."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gpu_frame(engine, pos, w, width, height, size_scale, limits):
    import torch

    board = torch.full((engine.frame_bytes(width, height),), 7, dtype=torch.uint8, device="cuda")
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1, 2)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda()
    engine.display(p, m, width, height, size_scale, limits, board, num_star=len(m))
    torch.cuda.synchronize()
    return board.cpu().numpy()


def test_display_matches_reference_frames(engine, display_golden):
    for c in display_golden:
        frame = gpu_frame(engine, c["pos"], c["w"], c["width"], c["height"], c["size_scale"], c["limits"])
        np.testing.assert_array_equal(frame, c["frame"])


@pytest.mark.parametrize("n,width,height,size_scale", [
    (1 << 20, 1920, 1080, 0.002),
    (3_000_000, 1024, 768, 0.0005),
    (100_003, 37, 23, 0.01),
])
def test_display_matches_oracle_large(engine, orc, n, width, height, size_scale):
    rng = np.random.default_rng(n)
    r = np.sqrt(rng.uniform(0.0, 1.0, n))
    a = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([1.1 * r * np.cos(a), 0.8 * r * np.sin(a)], 1).astype(np.float32)
    w = (rng.uniform(0, 9, n) * size_scale) ** 2
    limits = (-1.0, -0.75, 1.0, 0.75)
    frame = gpu_frame(engine, pos, w, width, height, size_scale, limits)
    np.testing.assert_array_equal(frame, orc.display(pos, w, width, height, size_scale, limits))


@pytest.mark.parametrize("width,height,n", [
    (3840, 2160, 2_000_000),  # the bitmask raster over 6 bands
    (6000, 4500, 20_000),     # more bits than 16 shared-memory bands: the byte-store raster
])
def test_display_large_frames(engine, orc, width, height, n):
    rng = np.random.default_rng(width)
    pos = rng.uniform(-1.05, 1.05, (n, 2)).astype(np.float32)
    pos[:64, 1] = 1.0 - rng.uniform(0, 3e-3, 64)  # stars on the top rows
    pos[64:128, 1] = -1.0 - rng.uniform(0, 4e-4, 64)  # and on row `height`
    w = (rng.uniform(0, 9, n) * 0.01) ** 2
    frame = gpu_frame(engine, pos, w, width, height, 0.01, (-1, -1, 1, 1))
    np.testing.assert_array_equal(frame, orc.display(pos, w, width, height, 0.01, (-1, -1, 1, 1)))


def test_display_unaligned_frame(engine, orc):
    """A frame that does not start on a 16-byte boundary takes the byte-wise stores of the expansion."""
    import torch

    rng = np.random.default_rng(5)
    n, width, height = 50_000, 200, 120
    pos = rng.uniform(-1.0, 1.0, (n, 2)).astype(np.float32)
    w = (rng.uniform(0, 9, n) * 0.01) ** 2
    fb = engine.frame_bytes(width, height)
    buf = torch.full((fb + 3,), 7, dtype=torch.uint8, device="cuda")
    p = torch.from_numpy(pos).cuda()
    m = torch.from_numpy(w.astype(np.float32)).cuda()
    engine.display(p, m, width, height, 0.01, (-1, -1, 1, 1), buf.data_ptr() + 3, num_star=n)
    torch.cuda.synchronize()
    out = buf.cpu().numpy()
    assert np.all(out[:3] == 7)
    np.testing.assert_array_equal(out[3:], orc.display(pos, w, width, height, 0.01, (-1, -1, 1, 1)))


def test_display_special_values_and_empty(engine, orc):
    pos = np.array([[np.nan, 0.0], [0.0, np.nan], [np.inf, 0.0], [-np.inf, 0.0], [1e30, 0.0], [0.0, -1e30],
                    [-0.75, -0.75], [0.3, 0.3], [0.999, -0.999], [-1.0, 1.0]], np.float32)
    w = np.array([1.0, 1.0, 1.0, 1.0, 1.0, 1.0, -4.0, np.inf, 100.0, 0.0], np.float32)
    for width, height in ((8, 8), (9, 7), (1, 1), (2, 3)):
        frame = gpu_frame(engine, pos, w, width, height, 1.0, (-1, -1, 1, 1))
        np.testing.assert_array_equal(frame, orc.display(pos, w, width, height, 1.0, (-1, -1, 1, 1)))
    empty = gpu_frame(engine, np.zeros((0, 2)), np.zeros(0), 16, 10, 1.0, (-1, -1, 1, 1))
    assert np.all(empty[:160] == 0) and np.all(empty[160:] == 128) and len(empty) == 240


def test_display_rejects_bad_arguments(engine):
    import torch

    board = torch.zeros(100, dtype=torch.uint8, device="cuda")
    p = torch.zeros((4, 2), device="cuda")
    m = torch.ones(4, device="cuda")
    for args in ((0, 8, 1.0, (-1, -1, 1, 1)), (8, 8, 0.0, (-1, -1, 1, 1)), (8, 8, 1.0, (1, -1, -1, 1))):
        with pytest.raises(engine.NbfmmError):
            engine.display(p, m, args[0], args[1], args[2], args[3], board, num_star=4)


def make_stars(engine, n, limits=(-1.0, -1.0, 1.0, 1.0), width=160, height=120, size_scale=0.01):
    import torch

    st = engine.Stars(3, n, width, height, 30, 1e-3, 1.0, size_scale, limits, (-1.2, -1.2, 1.2, 1.2),
                      epsilon=1e-2)
    rng = np.random.default_rng(n)
    cur = rng.uniform(-1.3, 1.3, (n, 2)).astype(np.float32)  # some start outside the position limits
    prev = (cur + rng.normal(scale=1e-3, size=(n, 2))).astype(np.float32)
    w = rng.uniform(0, 0.05, n).astype(np.float32) ** 2
    st.gpuptr_position_cur_.copy_(torch.from_numpy(cur))
    st.gpuptr_position_pre_.copy_(torch.from_numpy(prev))
    st.gpuptr_weight_.copy_(torch.from_numpy(w))
    torch.cuda.synchronize()
    return st, cur, prev, w


def test_stars_display_draws_then_prunes(engine, orc):
    import torch

    n = 20_000
    st, cur, prev, w = make_stars(engine, n)
    board = torch.empty(engine.frame_bytes(160, 120), dtype=torch.uint8, device="cuda")
    st.display(board)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(board.cpu().numpy(), orc.display(cur, w, 160, 120, 0.01, (-1.2, -1.2, 1.2, 1.2)))
    kept = orc.prune(cur, prev, w, (-1.0, -1.0, 1.0, 1.0))
    assert st.num_star_ == kept
    np.testing.assert_array_equal(st.gpuptr_position_cur_.cpu().numpy(), cur)
    np.testing.assert_array_equal(st.gpuptr_position_pre_.cpu().numpy(), prev)
    np.testing.assert_array_equal(st.gpuptr_weight_.cpu().numpy(), w)
    # A second prune keeps everything.
    st.prune()
    assert st.num_star_ == kept


def test_stars_display_after_updates_and_prune(engine, orc):
    import torch

    st, _, _, _ = make_stars(engine, 8192)
    board = torch.empty(engine.frame_bytes(160, 120), dtype=torch.uint8, device="cuda")
    st.display(board)
    for _ in range(3):
        st.update(2)
        n = st.num_star_
        cur = st.gpuptr_position_cur_.cpu().numpy()[:n]
        w = st.gpuptr_weight_.cpu().numpy()[:n]
        st.display(board)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(board.cpu().numpy(), orc.display(cur, w, 160, 120, 0.01, (-1.2, -1.2, 1.2, 1.2)))
        assert st.num_star_ == n  # update already pruned


def test_movie_file_matches_frames(engine, orc, tmp_path):
    import torch

    n, width, height, frames = 6000, 96, 64, 5
    st, _, _, _ = make_stars(engine, n, width=width, height=height)
    path = os.path.join(str(tmp_path), "stars.y4m")
    expected = []
    with engine.Movie(st, path) as mv:
        for k in range(frames):
            if k:
                st.update(1)
            torch.cuda.synchronize()
            m = st.num_star_
            expected.append(orc.display(st.gpuptr_position_cur_.cpu().numpy()[:m], st.gpuptr_weight_.cpu().numpy()[:m],
                                        width, height, 0.01, (-1.2, -1.2, 1.2, 1.2)))
            mv.frame()
    data = open(path, "rb").read()
    header = f"YUV4MPEG2 W{width} H{height} F30:1 Ip A1:1 C420\n".encode()
    assert data.startswith(header)
    fb = width * height * 3 // 2
    body = data[len(header):]
    assert len(body) == frames * (6 + fb)
    for k in range(frames):
        chunk = body[k * (6 + fb):(k + 1) * (6 + fb)]
        assert chunk[:6] == b"FRAME\n"
        np.testing.assert_array_equal(np.frombuffer(chunk[6:], np.uint8), expected[k], err_msg=f"frame {k}")

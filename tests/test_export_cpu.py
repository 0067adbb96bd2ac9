"""CPU checks of the framebuffer export helpers and of the oracle's
restatement of the reference's display shader and trace/statistics formats."""
import numpy as np

from oracle import oracle


def test_display_known_answers():
    W, H = 16, 8
    col = np.zeros((W * H, 4), np.float32)
    # tiled layout: pixel (x, y) -> ((x//8) + 2*(y//8))*64 + x%8 + 8*(y%8)
    def put(x, y, rgb):
        col[((x // 8) + 2 * (y // 8)) * 64 + (x % 8) + 8 * (y % 8), :3] = rgb
    put(0, 0, (0.5, 0.0, 1.0))      # bottom-left of the framebuffer
    put(15, 7, (2.0, 0.25, -0.0))   # top-right, over-range red
    img = oracle.display_image(col, W, H)
    assert img.shape == (H, W, 3)
    # 0.5^0.454545 = 0.7297 -> 186; 0 -> 0; 1 -> 255; 0.25^0.454545 = 0.5325 -> 136
    assert tuple(img[H - 1, 0]) == (186, 0, 255)          # bottom row is last
    assert tuple(img[0, W - 1]) == (255, 136, 0)           # top row is first


def test_ppm_pfm_round_trip(tmp_path):
    from micropolis_gb300.renderer import read_ppm, write_pfm, write_ppm
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(5, 7, 3), dtype=np.uint8)
    write_ppm(str(tmp_path / "a.ppm"), img)
    assert np.array_equal(read_ppm(str(tmp_path / "a.ppm")), img)
    f = rng.random((5, 7, 3)).astype(np.float32)
    write_pfm(str(tmp_path / "a.pfm"), f)
    data = (tmp_path / "a.pfm").read_bytes()
    assert data.startswith(b"PF\n7 5\n-1.0\n")
    assert np.array_equal(np.frombuffer(data[len(b"PF\n7 5\n-1.0\n"):], "<f4").reshape(5, 7, 3), f)


def test_trace_and_stats_parsers():
    items = oracle.parse_trace("dice@batched:10:10:12:40:3:1|2\nframe@plain:0:0:0:7:0:\n")
    assert items[0] == ("dice", "batched", 10, 10, 12, 40, 3, [1, 2])
    assert items[1][0] == "frame" and items[1][7] == []
    s = oracle.parse_stats("opencl_mem = 12;\nopencl_mem@framebuffer = 12;\nmax_patches = 3;\n"
                           "bound_n_split_balance = 4 5 6 ;")
    assert s == {"opencl_mem": 12, "opencl_mem@framebuffer": 12, "max_patches": 3,
                 "bound_n_split_balance": [4, 5, 6]}

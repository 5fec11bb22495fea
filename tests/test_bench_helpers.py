"""bench.py's host-side accounting, on the CPU: the emulated form's aux batches follow the
engine's rule, so the claimed kernel launches per build match the ncu launch list of the C2
workload (16 a build: J 6, digits of C 2, and per aux batch the half-transform, the split of X,
the contraction and the reduction), and the issued-flop count uses the engine's column chunks."""
import bench


def test_aux_batches_and_launches(monkeypatch):
    monkeypatch.delenv("GDFJK_OZ_XCAP_GB", raising=False)
    # C2: nocc_p 160, groups of 6 aux functions, 24 GB of X buffers -> 3594-row batches
    assert bench.oz_aux_batches(1856, 4448, 160) == 2
    assert bench.build_launches(1856, 4448, 160, emulated=True) == 16
    assert bench.build_launches(1856, 4448, 160, emulated=False) == 10
    # C4 and the 128-row profiling case fit one batch
    assert bench.build_launches(384, 1856, 80, emulated=True) == 12
    assert bench.build_launches(1856, 128, 160, emulated=True) == 12
    # a smaller X budget gives more batches, never fewer rows than a group
    monkeypatch.setenv("GDFJK_OZ_XCAP_GB", "0.002")
    assert bench.oz_aux_batches(384, 1856, 80) == -(-1856 // 10)  # nocc_p 96: groups of 10
    monkeypatch.setenv("GDFJK_OZ_XCAP_GB", "nonsense")
    assert bench.oz_aux_batches(1856, 4448, 160) == 2


def test_issued_flops_use_the_engine_chunks():
    # nocc 160: two column chunks of 80; nbf 1856 padded to 1920
    assert bench.oz_issued_flops(1856, 4448, 160) == 28 * 2.0 * 4448 * 1920 * 1920 * 160
    # nocc 100 -> nocc_p 128: two chunks of 64
    assert bench.oz_issued_flops(1856, 10, 100) == 28 * 2.0 * 10 * 1920 * 1920 * 128

"""Failure detection on the GPU without a fault: a dependency wait that nothing will
ever satisfy (a job naming itself as its parent job, which only the unvalidated
device-job entry accepts) gives up after its poll limit, records TP_E_TIMEOUT in the
status word, and the launch still ends; the context stays usable and the next batch
produces correct tiles."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dependency_wait_gives_up_with_a_status(gpu, oracle_lib):
    import torch
    tp = gpu
    W = 101
    rng = np.random.default_rng(3)
    parent = (rng.standard_normal((1, W, W)) * 300.0).astype(np.float32)
    elev = tp.TileStorage(W, 3, 4)
    elev.upload(2, tp.ZF, parent)
    elev.upload(2, tp.ZM, np.maximum(parent, np.float32(0.0)))
    tp.stream_check()
    job = tp.make_job(1, 1, 0, out_slot=0, parent_slot=2, tile_meters=5000.0, parent_job=0)  # waits on itself
    arr = (tp.TileJob * 1)(job)
    dev = torch.empty(C.sizeof(arr), dtype=torch.uint8, device="cuda")
    dev.copy_(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8))
    torch.cuda.synchronize()
    frame = tp.Frame()
    frame.add_device(elev, None, None, tp.make_params(), C.c_void_p(dev.data_ptr()), 1, has_dependencies=True)
    frame.launch()
    with pytest.raises(tp.TPError) as err:
        tp.stream_check()
    assert err.value.code == tp.TP_E_TIMEOUT
    tp.stream_check()  # the status word was read and cleared
    frame.close()
    # the same tile through a valid batch: correct, and no status left behind
    tp.elevation_batch(elev, None, None, tp.make_params(),
                       [tp.make_job(1, 1, 0, out_slot=1, parent_slot=2, tile_meters=5000.0)])
    tp.stream_check()
    zf, _, _ = oracle_lib.elevation_tile(W, 1, 1, 0, parent[0], np.maximum(parent[0], 0), None)
    assert np.array_equal(elev.download(1, 1, tp.ZF)[0], zf)

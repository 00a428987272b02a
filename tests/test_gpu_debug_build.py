"""The debug build (libproland_gb300_debug.so, PROLAND_GB300_DEBUG=1) on the GPU, in a
subprocess: it produces the oracle's tiles with every storage's guard regions intact;
and jobs of a device job array that the host cannot validate -- an output slot past
the capacity the checks use (lowered with tp_debug_check_capacity, so that the slot
still lies inside the allocation), a job naming itself as its parent -- are reported
as TP_E_BOUNDS and skipped by the frame and ortho kernels while the other jobs are
produced as usual."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import ctypes as C
import sys
sys.path.insert(0, ROOT); sys.path.insert(0, ROOT + "/proland-4.0_gb300"); sys.path.insert(0, ROOT + "/tests")
import numpy as np
import torch
import oracle
import proland_gb300 as tp
from tilecase import smooth_tile

L = tp.lib()
assert L.tp_build_is_debug() == 1, tp._lib.LIB_PATH
W, n = 101, 8
rng = np.random.default_rng(5)
elev, res, nrm = tp.TileStorage(W, 3, 16), tp.TileStorage(W, 1, 8), tp.TileStorage(W - 4, 2, 16)
parent = smooth_tile(W, 9)
elev.upload(8, tp.ZF, parent[None])
elev.upload(8, tp.ZM, np.maximum(parent, 0)[None])
resid = (rng.standard_normal((n, W, W)) * 40.0).astype(np.float32)
res.upload(0, 0, resid)
table = oracle.dem_noise(W)
jobs = []
for k in range(n):
    tx, ty = 4 + (k & 1), 6 + ((k >> 1) & 1)
    rot, layer = tp.noise_select(1, 3, tx, ty)
    jobs.append(tp.make_job(3, tx, ty, out_slot=k, parent_slot=8, residual_slot=k, normal_slot=k, noise_rot=rot,
                            noise_layer=layer, noise_amp=-20.0, tile_meters=5000.0))
params = tp.make_params()


def want(k):
    j = jobs[k]
    return oracle.elevation_tile(W, 3, j.tx, j.ty, parent, np.maximum(parent, 0), resid[k], noise=table[j.noise_layer],
                                 noise_rot=j.noise_rot, noise_amp=j.noise_amp)[0]


# 1. a correct batch
tp.elevation_batch(elev, res, nrm, params, jobs)
tp.stream_check()
zf = elev.download(0, n, tp.ZF)
assert all(np.array_equal(zf[k], want(k)) for k in range(n)), "debug build differs from the oracle"
for s in (elev, res, nrm):
    assert L.tp_storage_check_guards(s.handle) == 0, tp.lib().tp_last_error()

# 2. planted bad jobs in a device job array: slot 13 is past the checked capacity (12)
# but inside the allocation (16 slots); job 5 names itself as its parent
tp.check(L.tp_debug_check_capacity(elev.handle, 12))
bad = [tp.TileJob.from_buffer_copy(j) for j in jobs]
bad[3].out_slot = 13
bad[5].parent_job = 5
sentinel = np.full((1, W, W), 12345.0, np.float32)
elev.upload(13, tp.ZF, sentinel)
for k in range(n):
    elev.upload(k, tp.ZF, np.zeros((1, W, W), np.float32))
arr = (tp.TileJob * n)(*bad)
dev = torch.empty(C.sizeof(arr), dtype=torch.uint8, device="cuda")
dev.copy_(torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8))
torch.cuda.synchronize()
tp.elevation_batch_device(elev, res, nrm, params, C.c_void_p(dev.data_ptr()), n)
try:
    tp.stream_check()
    raise AssertionError("no TP_E_BOUNDS reported")
except tp.TPError as e:
    assert e.code == tp.TP_E_BOUNDS, e
zf = elev.download(0, 16, tp.ZF)
assert np.array_equal(zf[13], sentinel[0]), "the out-of-range slot was written"
for k in range(n):
    if k in (3, 5):
        assert not zf[k].any(), "a rejected job was produced"
    else:
        assert np.array_equal(zf[k], want(k)), k
for s in (elev, res, nrm):
    assert L.tp_storage_check_guards(s.handle) == 0, tp.lib().tp_last_error()
tp.check(L.tp_debug_check_capacity(elev.handle, 0))

# 3. the ortho kernel: output slot 6 past the checked capacity 4 of an 8-slot storage
OW = 196
orth, ores = tp.TileStorage(OW, 1, 8), tp.TileStorage(OW, 1, 8)
tp.check(L.tp_debug_check_capacity(orth.handle, 4))
opar = tp.make_ortho_params(root_color=(0.2, 0.5, 0.1, 1.0), noise_color=(0.3, 0.3, 0.4, 1.0), scale=2.0, hsv=False)
ojobs = [tp.make_ortho_job(0, 0, 0, out_slot=k, parent_slot=-1, residual_slot=-1, noise_rot=0, noise_layer=k % 6,
                           noise_amp=255.0) for k in range(3)]
ojobs[1].out_slot = 6
oarr = (tp.OrthoJob * 3)(*ojobs)
odev = torch.empty(C.sizeof(oarr), dtype=torch.uint8, device="cuda")
odev.copy_(torch.frombuffer(bytearray(bytes(oarr)), dtype=torch.uint8))
torch.cuda.synchronize()
tp.ortho_batch_device(orth, ores, opar, C.c_void_p(odev.data_ptr()), 3)
try:
    tp.stream_check()
    raise AssertionError("no TP_E_BOUNDS reported by the ortho kernel")
except tp.TPError as e:
    assert e.code == tp.TP_E_BOUNDS, e
tiles = orth.download(0, 8, 0)
assert not tiles[6].any() and tiles[0].any() and tiles[2].any()
assert L.tp_storage_check_guards(orth.handle) == 0
print("debug build ok")
'''


def test_debug_build_checks_and_guards(gpu):
    out = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + SCRIPT], cwd=ROOT,
                         env=dict(os.environ, PROLAND_GB300_DEBUG="1"), capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, (out.stdout[-2000:], out.stderr[-3000:])
    assert "debug build ok" in out.stdout

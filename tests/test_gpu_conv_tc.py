"""The tcgen05 convolution of the learned warm start (k_conv32_tc,
iskra_gb300/csrc/lws.cu) against the mma.sync kernel it replaced
(k_conv32, selected by ISKRA_CONV_MMA_SYNC=1): the forward pass and every
parameter gradient of the network on the 1024 x 1024 image of the 2D
discharge and on a 104 x 72 image (16-row tiles cut by the image edge at
every level, 8-pixel tiles at levels 1 to 3).  Both kernels accumulate the
K = 16 slices in FP32 in the same (tap, slice) order, so the forward pass
agrees bit for bit in practice (measured at 1024 x 1024); the weight
gradient adds its per-block sums with atomics in any order.  Tolerances:
1e-2 (relative L2) on y and on the gradient.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, {root!r})
from iskra_gb300.device import Context
ny, nx = {ny}, {nx}
ctx = Context(nx, ny, 1e-4, 1e-4, (0, 0, 0, 0))
ctx.lws_create(0, seed=3)
rng = np.random.default_rng(11)
x = rng.standard_normal((ny, nx)).astype(np.float32)
t = (0.1 * rng.standard_normal((ny, nx))).astype(np.float32)
y = ctx.lws_forward(x)
loss, g = ctx.lws_loss_grad(x, t)
ctx.close()
np.savez({out!r}, y=y, g=g, loss=loss)
"""


def _run(tmp_path, ny, nx, legacy):
    out = str(tmp_path / f"conv_{ny}x{nx}_{int(legacy)}.npz")
    env = dict(os.environ)
    env.pop("ISKRA_CONV_MMA_SYNC", None)
    if legacy:
        env["ISKRA_CONV_MMA_SYNC"] = "1"
    code = SCRIPT.format(root=ROOT, ny=ny, nx=nx, out=out)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


@pytest.mark.parametrize("ny,nx", [(1024, 1024), (104, 72)])
def test_tcgen05_conv_matches_mma_sync(tmp_path, ny, nx):
    tc = _run(tmp_path, ny, nx, legacy=False)
    ms = _run(tmp_path, ny, nx, legacy=True)
    ry = np.linalg.norm(tc["y"] - ms["y"]) / np.linalg.norm(ms["y"])
    rg = np.linalg.norm(tc["g"] - ms["g"]) / np.linalg.norm(ms["g"])
    print(f"{ny}x{nx}: y rel {ry:.2e}, gradient rel {rg:.2e}, loss {float(tc['loss']):.6e} vs {float(ms['loss']):.6e}")
    assert np.all(np.isfinite(tc["y"])) and np.all(np.isfinite(tc["g"]))
    assert ry <= 1e-2, ry
    assert rg <= 1e-2, rg
    assert abs(float(tc["loss"]) - float(ms["loss"])) <= 1e-2 * float(ms["loss"])

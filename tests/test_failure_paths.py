"""Failure detection without a GPU fault: a bounded device wait that nothing
ends gives up and reports MYPBR_ERR_DEVICE_TIMEOUT, after which the context
still renders; without a GPU the same call reports MYPBR_ERR_NO_DEVICE.
Queue overflow cannot happen by construction (every queue holds a wave's
slots), and malformed inputs are rejected before any launch (tests of the
host layer and of damaged files)."""
import numpy as np
import pytest
import torch

import mypbr_gb300 as mp
from conftest import scene_path


def test_wait_timeout_without_a_gpu():
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert mp.lib().mypbr_gpu_test_wait_timeout() == 9


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_the_context_survives():
    status = mp.lib().mypbr_gpu_test_wait_timeout()
    assert status == 4, mp.lib().mypbr_last_error()
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    G = mp.GpuScene(sc)
    cam = sc.camera
    cam.image_width = 16
    cam.samples_per_pixel = 4
    rad = cam.render(G).radiance
    assert np.isfinite(rad).all() and rad.mean() > 0

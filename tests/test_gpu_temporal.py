"""Temporal reprojection (trace.frag:275-322, renderer.ts:441-451, 717-731):
after a camera move the first traced sample starts from the previous view's
averages reprojected onto the new view; compared per pixel with the oracle's
restatement fed the same previous targets."""
import copy

import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu

W_, H_ = 64, 48


def _moved(cam, dx, dyaw):
    c = copy.deepcopy(cam)
    c.position = (cam.position[0] + dx, cam.position[1], cam.position[2])
    c.target = (cam.target[0] + dyaw, cam.target[1], cam.target[2])
    return c


@pytest.mark.parametrize("dx,dyaw", [(0.05, 0.0), (0.2, 0.1)])
def test_reprojected_sample_matches_oracle(dx, dyaw):
    sc = W.box_scene(3, 3)
    r = Renderer(W_, H_)
    r.settings.max_bounces = 6
    r.load_scene(sc)
    r.trace_samples(8)
    prev = r.read()
    cam2 = _moved(sc.camera, dx, dyaw)
    r.upload_camera(cam2)  # temporal on: the history is kept
    r.trace_samples(1)
    col, alb, nrm, hist = r.read()
    assert r.samples() == 9
    prep = OR.prepare(sc)
    oc, oa, on, oh = OR.render_reproject(prep, OR.camera_of(cam2), W_, H_, 8, 1, OR.camera_of(sc.camera), prev,
                                         max_bounces=6)
    assert (hist == oh).mean() > 0.99
    reused = hist > 1.5
    assert 0.2 < reused.mean() < 1.0  # some history survives, some pixels are disoccluded
    assert hist.max() <= 9.0 + 1e-6  # at most HISTORY_CAP reprojected samples, plus the new one
    close = np.abs(col[..., :3] - oc[..., :3]) <= 1e-3 * (np.abs(oc[..., :3]) + 1e-3)
    assert close.mean() > 0.97, close.mean()
    r.dispose()


def test_temporal_off_restarts_the_average():
    sc = W.box_scene(3, 3)
    r = Renderer(W_, H_)
    r.settings.temporal = False
    r.load_scene(sc)
    r.trace_samples(4)
    r.upload_camera(_moved(sc.camera, 0.05, 0.0))
    r.trace_samples(1)
    assert r.samples() == 1 and np.all(r.read()[3] == 1.0)
    r.dispose()

"""Frame constants: the UniformBufferObject build of the reference, restated.

NextEngine::GetUniformBufferObject (src/Runtime/Engine.cpp:736-849) fills the camera
matrices with glm (perspective with a [0,1] depth range, right-handed, Y flipped for
Vulkan, Halton TAA jitter in Projection[2][0..1]), keeps last frame's view-projection for
motion vectors, and copies the user settings. glm is an un-vendored dependency of the
reference (vcpkg), so its perspectiveRH_ZO / lookAtRH / inverse are restated from their
published formulas here in float64 and rounded once to float32.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi


def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


def look_at(eye, center, up) -> np.ndarray:
    """glm::lookAtRH, returned as a 4x4 numpy matrix (row = math row)."""
    eye = np.asarray(eye, np.float64)
    f = _normalize(np.asarray(center, np.float64) - eye)
    s = _normalize(np.cross(f, up))
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -np.dot(s, eye)
    m[1, 3] = -np.dot(u, eye)
    m[2, 3] = np.dot(f, eye)
    return m


def perspective_zo(fovy_rad: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    """glm::perspectiveRH_ZO (math row/col indexing)."""
    t = math.tan(fovy_rad / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = zfar / (znear - zfar)
    m[3, 2] = -1.0
    m[2, 3] = -(zfar * znear) / (zfar - znear)
    return m


def halton(index: int, base: int) -> float:
    f, r = 1.0, 0.0
    while index > 0:
        f /= base
        r += f * (index % base)
        index //= base
    return r


def _cm(m: np.ndarray):
    """4x4 math matrix -> column-major float[16] (glm memory order)."""
    return np.asarray(m, dtype=np.float64).T.reshape(-1).astype(np.float32)


class Camera:
    def __init__(self, eye, center, up=(0.0, 1.0, 0.0), fov_deg=40.0, aperture=0.0, focus_distance=10.0):
        self.eye = np.asarray(eye, np.float64)
        self.center = np.asarray(center, np.float64)
        self.up = np.asarray(up, np.float64)
        self.fov_deg = float(fov_deg)
        self.aperture = float(aperture)
        self.focus_distance = float(focus_distance)

    def model_view(self) -> np.ndarray:
        return look_at(self.eye, self.center, self.up)

    def orbit(self, degrees: float) -> "Camera":
        """Rotate the eye about the vertical axis through `center` (motion benchmark orbit,
        src/Application/gkNextBenchmark/gkNextMotionBenchmark.cpp:50-51)."""
        a = math.radians(degrees)
        c, s = math.cos(a), math.sin(a)
        rel = self.eye - self.center
        x = c * rel[0] + s * rel[2]
        z = -s * rel[0] + c * rel[2]
        return Camera(self.center + np.array([x, rel[1], z]), self.center, self.up, self.fov_deg,
                      self.aperture, self.focus_distance)


class Settings:
    """User settings that reach the UBO (the UserSettings fields of src/Runtime/Engine.cpp:111-163).
    The defaults here are a light test setting (1 sample, 4 bounces, no TAA); the scene
    constructors set their configuration's values, and reference_defaults() gives the
    reference's own."""

    def __init__(self, samples=1, bounces=4, max_bounces=10, temporal_frames=16, taa=False,
                 bf_size=5, bf_sigma=2.0, bf_sigma_lum=3.0, bf_sigma_normal=0.005, paper_white_nit=600.0,
                 has_sky=False, sky_color=(0.0, 0.0, 0.0, 1.0), sky_intensity=1.0, has_sun=False,
                 sun_direction=(0.0, 1.0, 0.0), sun_intensity=0.0, progressive=False, fast_gather=False,
                 hdr=False, denoiser=abi.DENOISE_JBF, nee_mode=abi.NEE_REFERENCE, flags=0, sky_texture=None,
                 sky_rotation=0.0):
        self.__dict__.update(locals())
        del self.__dict__["self"]

    @classmethod
    def reference_defaults(cls) -> "Settings":
        """The reference's startup values: the command-line defaults (8 samples, 5 bounces, 10 at
        most, 16 temporal frames; src/Options.cpp:11-14) and TAA on, the bilateral filter's
        2.0 / 3.0 / 0.005 with size 5, 600-nit paper white (src/Runtime/Engine.cpp:111-163)."""
        return cls(samples=8, bounces=5, max_bounces=10, temporal_frames=16, taa=True)


class FrameBuilder:
    """Builds one GkrtFrameConstants per frame, keeping last frame's matrices
    (prevUBO_ in NextEngine::GetUniformBufferObject)."""

    def __init__(self, width: int, height: int, settings: Settings):
        self.width, self.height = int(width), int(height)
        self.s = settings
        self.prev_vp = None
        self.prev_vp_unjit = None
        self.prev_total_frames = 0      # TotalFrames of the previous UBO (zero before the first)
        self.total_frames = 0

    def build(self, cam: Camera, total_frames: int | None = None) -> abi.GkrtFrameConstants:
        s = self.s
        if total_frames is None:
            total_frames = self.total_frames
        W, H = self.width, self.height
        mv = cam.model_view()
        proj = perspective_zo(math.radians(cam.fov_deg), W / float(H), 0.2, 2000.0)
        proj[1, 1] *= -1.0
        proj_unjit = proj.copy()
        if s.taa:
            n = max(1, int(s.temporal_frames))
            jx = halton(total_frames % n + 1, 2) - 0.5
            jy = halton(total_frames % n + 1, 3) - 0.5
            proj[0, 2] = jx / W * 2.0   # glm Projection[2][0]
            proj[1, 2] = jy / H * 2.0   # glm Projection[2][1]
        vp = proj @ mv
        vp_unjit = proj_unjit @ mv
        fc = abi.GkrtFrameConstants()
        fc.model_view[:] = _cm(mv)
        fc.projection[:] = _cm(proj)
        fc.model_view_inverse[:] = _cm(np.linalg.inv(mv))
        fc.projection_inverse[:] = _cm(np.linalg.inv(proj))
        fc.view_projection[:] = _cm(vp)
        fc.view_projection_unjit[:] = _cm(vp_unjit)
        # last frame's matrices only when last frame's TotalFrames was not zero (Engine.cpp:786-787):
        # the first frame, and the one after it, see no camera motion
        keep = self.prev_vp is not None and self.prev_total_frames != 0
        prev = self.prev_vp if keep else vp
        prevu = self.prev_vp_unjit if keep else vp_unjit
        fc.prev_view_projection[:] = _cm(prev)
        fc.prev_view_projection_unjit[:] = _cm(prevu)
        sd = _normalize(s.sun_direction)
        fc.sun_direction[:] = [sd[0], sd[1], sd[2], 0.0]
        fc.sun_color[:] = [s.sun_intensity, s.sun_intensity, s.sun_intensity, 0.0]
        fc.sky_color[:] = list(s.sky_color)
        fc.aperture = cam.aperture
        fc.focus_distance = cam.focus_distance
        fc.paper_white_nit = s.paper_white_nit
        fc.sky_intensity = s.sky_intensity
        fc.total_frames = total_frames
        fc.number_of_samples = s.samples
        fc.number_of_bounces = s.bounces
        fc.max_number_of_bounces = s.max_bounces
        fc.temporal_frames = 256 if s.progressive else s.temporal_frames
        fc.has_sky = 1 if s.has_sky else 0
        fc.has_sun = 1 if (s.has_sun and s.sun_intensity > 0) else 0
        fc.taa = 1 if s.taa else 0
        fc.fast_gather = 1 if s.fast_gather else 0
        fc.progressive_render = 1 if s.progressive else 0
        fc.bf_size = s.bf_size
        fc.hdr = 1 if s.hdr else 0
        fc.bf_sigma = s.bf_sigma
        fc.bf_sigma_lum = s.bf_sigma_lum
        fc.bf_sigma_normal = s.bf_sigma_normal
        fc.denoiser = s.denoiser
        fc.nee_mode = s.nee_mode
        fc.flags = s.flags
        if getattr(s, "sky_texture", None) is not None:   # the HDR sky (SkyIdx, SkyRotation)
            fc.flags |= abi.FRAME_SKY_TEXTURE
            fc.sky_index = int(s.sky_texture)
            fc.sky_rotation = float(getattr(s, "sky_rotation", 0.0))
        self.prev_vp, self.prev_vp_unjit = vp, vp_unjit
        self.prev_total_frames = total_frames
        self.total_frames = total_frames + 1
        return fc

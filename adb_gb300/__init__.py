"""abd_gb300 — GB300-native affine-body contact step (IPC barrier + friction + CCD +
line search) behind a C ABI, a drop-in for the reference's ABD::implicit_euler."""
from .scene import Config, Scene, load_config, load_scene  # noqa: F401

__all__ = ["Config", "Scene", "load_config", "load_scene", "ABD"]


def __getattr__(name):
    if name == "ABD":
        from .abd import ABD
        return ABD
    raise AttributeError(name)

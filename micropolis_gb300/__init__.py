"""GB300-native REYES core: bound-and-split, dice, shade and rasterize of
bicubic Bezier and Gregory patches on one GPU, behind the reference's
Renderer interface (see renderer.Renderer) and a C ABI (include/mp_core.h)."""
from .options import ReyesOptions, load_options  # noqa: F401
from . import scenes  # noqa: F401


def __getattr__(name):
    # the renderer loads libmpcore.so; import it lazily so that options and
    # scenes stay usable before the library is built
    if name in ("Renderer", "Projection", "render_scene", "renderer_for"):
        from . import renderer
        return getattr(renderer, name)
    raise AttributeError(name)

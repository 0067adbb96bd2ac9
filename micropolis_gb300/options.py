"""REYES options with the reference's names and defaults.

Defaults are the values of the reference's reyes.options (the schema
defaults in src/Reyes/config.xml:42-142 differ and are not used).  The same
`key = value` file format (`//` comments, `#hash:` trailer) and `--key=value`
command-line overrides (src/micropolis/main.cpp:489-576) are accepted.
"""
from __future__ import annotations

import dataclasses
import re


@dataclasses.dataclass
class ReyesOptions:
    window_size: tuple = (1600, 1200)          # reyes.options:2
    clear_color: tuple = (0.1, 0.1, 0.7, 0.0)  # reyes.options:11
    reyes_patch_size: int = 8                  # :14
    bound_n_split_limit: float = 8.0           # :17
    cull_ribbon: float = 32.0                  # :20
    backface_culling: bool = True              # :31
    bound_sample_rate: int = 3                 # :37 (the CPU criterion fixes 3)
    max_split_depth: int = 23                  # :40
    reyes_patches_per_pass: int = 100000       # :44
    framebuffer_tile_size: int = 8             # :47
    subpixel_bits: int = 6                     # :50
    dice_group_width: int = 8                  # :53
    displacement: bool = False                 # :67
    displacement_amplitude: float = 1.0        # multiplier on the hard-coded amplitudes
    batch_views: int = 1                       # framebuffer layers (batched views)
    path: str = "batched"                      # "plain" (per-pass) or "batched"
    queue_capacity: int = 0                    # first-frame capacities (0 = automatic; they grow)
    subpatch_capacity: int = 0
    spin_limit: int = 0                        # bounded-wait iterations (0 = default)
    overlap: bool = False                      # batched: rasterize while bound-and-split emits
    bns_blocks: int = 0                        # batched overlap: blocks starting with bound-and-split (0 = auto)
    raster_tile: int = 0                       # depth|id key buffer tile in pixels (0 = 8)
    dice_group: int = 0                        # sub-patches per fused block (0 = default)
    bound_criterion: int = 0                   # 0: the reference's CPU criterion, 1: its GPU criterion

    def update(self, **kw) -> "ReyesOptions":
        for k, v in kw.items():
            if not hasattr(self, k):
                raise KeyError(f"unknown option {k!r}")
            setattr(self, k, _coerce(getattr(self, k), v))
        return self


def _coerce(old, v):
    if isinstance(v, str):
        s = v.strip()
        if isinstance(old, bool):
            if s in ("true", "1"):
                return True
            if s in ("false", "0"):
                return False
            raise ValueError(f"bad bool {v!r}")
        if isinstance(old, tuple):
            parts = s.split()
            return tuple(type(old[0])(p) for p in parts)
        if isinstance(old, int):
            return int(s)
        if isinstance(old, float):
            return float(s)
        return s
    if isinstance(old, tuple):
        return tuple(v)
    if isinstance(old, bool):
        return bool(v)
    return type(old)(v)


_LINE = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*=\s*(.*?)\s*$")


def parse_options_text(text: str) -> dict:
    """Parse the reference's `.options` format into {key: string}."""
    out = {}
    for line in text.splitlines():
        line = line.split("//", 1)[0]
        if not line.strip() or line.lstrip().startswith("#"):
            continue
        m = _LINE.match(line)
        if m:
            out[m.group(1)] = m.group(2)
    return out


def parse_cli(argv) -> dict:
    """`--key=value` overrides, as src/micropolis/main.cpp:570-573 reads them."""
    out = {}
    for a in argv:
        if a.startswith("--") and "=" in a:
            k, v = a[2:].split("=", 1)
            out[k] = v
    return out


def load_options(text: str | None = None, argv=()) -> ReyesOptions:
    opts = ReyesOptions()
    known = {f.name for f in dataclasses.fields(ReyesOptions)}
    for src in (parse_options_text(text) if text else {}, parse_cli(argv)):
        opts.update(**{k: v for k, v in src.items() if k in known})
    return opts

"""Row-band sharding of one scene over several GPUs (one process per GPU).

Pixels are independent given their windows, so a scene splits into bands of
rows with no data-path collective: rank k computes rows [r0, r1) from the
stack rows [s0, s1), its band plus an apron of at least Ny rows on each side
(the reference's block overlap, src/evd/evd.cpp:419-443).  s0 is rounded
down to the 8-row tile grid of the mixed form, so a band's results are the
same bits as the whole scene's rows.  Gathering the bands (if a caller wants
one array) is the caller's business: the outputs of the ranks are disjoint.
"""
from dataclasses import dataclass


@dataclass(frozen=True)
class Band:
    r0: int      # first output row (scene coordinates)
    r1: int      # end of the output rows
    s0: int      # first stack / nmap row the rank holds
    s1: int      # end of the rows it holds

    @property
    def local_rows(self):
        """Output rows in the coordinates of the held rows."""
        return self.r0 - self.s0, self.r1 - self.s0


def row_bands(rows, world, half_window_y, align=8):
    """Bands of `rows` scene rows for `world` ranks: equal shares (multiples
    of `align` except the last), each with its apron."""
    if rows <= 0 or world <= 0:
        raise ValueError("rows and world must be positive")
    share = -(-rows // world)
    share = -(-share // align) * align
    bands = []
    for k in range(world):
        r0 = min(rows, k * share)
        r1 = min(rows, r0 + share)
        s0 = max(0, (r0 - half_window_y) // align * align)
        s1 = min(rows, r1 + half_window_y)
        bands.append(Band(r0, r1, s0, s1))
    return bands


def phase_link_band(stack, nmap, half_window, band, **kw):
    """Phase-link one band: `stack` / `nmap` hold the scene rows
    [band.s0, band.s1) (band-planar stack [N, s1-s0, cols]); returns the
    outputs of those rows with rows [r0, r1) computed."""
    from .linker import phase_link
    if band.r1 <= band.r0:
        return None
    return phase_link(stack, nmap, half_window, rows=band.local_rows, **kw)

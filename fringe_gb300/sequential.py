"""Sequential estimator: ministacks, compressed SLCs and the datum connection.

The reference's driver (src/sequential/sequential.py:147-254 with
src/sequential/Stack.py) walks the dates in ministacks of ``miniStackSize``.
Ministack k (1-based) is phase linked with ``miniStackCount = k`` over the
compressed SLCs of ministacks 1..k-1 followed by its own dates, so its phases
are referenced to its first own date and its compressed SLC sums only its own
dates (src/evd/evd.cpp:738-762).  The compressed SLCs of all ministacks are
then phase linked once more with ``miniStackCount = 1``: the datum
connection.  python/adjustMiniStacks.py:203-223 finally multiplies the phase
of every date by the datum phase of its ministack's compressed SLC.

Two entry points:

``sequential(stack, nmap, half_window, ...)``
    in memory.  The stack, the compressed SLCs and every intermediate stay on
    the GPU; each ministack is one ``phase_link`` call (fpl_run_async) on the
    caller's stream, the adjustment one ``fpl_adjust_wrapped`` launch.

``main(argv)`` / ``python -m fringe_gb300.sequential``
    file level, with the reference's command line (sequential.py:9-41) and
    its folder layout: ``fullStack/``, ``miniStacks/<first>_<last>/`` (stack
    VRTs and ``EVD/``), ``compressedSlc/<date>/<date>.slc`` and
    ``Datum_connection/``; each ministack runs through ``evdlib.Evd``
    (fpl_process).
"""
import argparse
import ctypes
import glob
import os
import re

import numpy as np

from . import _lib


def ministack_plan(ndates, mini_stack_size):
    """[(count, start, end)] of the loop in sequential.py:193-254: count is the
    1-based ministack number (miniStackCount), its own dates start..end-1."""
    if mini_stack_size < 1:
        raise ValueError("mini_stack_size must be >= 1")
    plan, count, start = [], 0, 0
    while start < ndates:
        count += 1
        end = min(start + mini_stack_size, ndates)
        plan.append((count, start, end))
        start += mini_stack_size
    return plan


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def sequential(stack, nmap, half_window, mini_stack_size=10, method="MLE", band_width=-1,
               min_neighbors=5, precision="fp32", adjust=True, device=0, ctx=None):
    """Sequential estimator over a stack held in memory.

    stack : complex64 [ndates, rows, cols]; nmap : uint32 [rows, cols, nulong]
            (NumPy arrays, copied to the GPU once, or CUDA torch tensors).
    Returns a dict of CUDA tensors (NumPy arrays for NumPy input):
      "ministacks": [dict(count, start, end, phase [k-1+n_k, rows, cols],
                     tcorr, comp)] -- the evd outputs of each ministack;
      "compressed": [nmini, rows, cols] compressed SLCs;
      "datum": dict(phase [nmini, rows, cols], tcorr, comp);
      "adjusted": [ndates, rows, cols] complex64 -- each date's ministack
                  phase times the datum phase of its ministack (adjust=True).
    """
    import torch
    from .linker import phase_link

    host = not _is_torch(stack)
    if host:
        dev = torch.device("cuda", device)
        S = torch.from_numpy(np.ascontiguousarray(stack, dtype=np.complex64)).to(dev)
        Nm = torch.from_numpy(np.ascontiguousarray(nmap).view(np.int32)).to(dev)
    else:
        if not stack.is_cuda:
            raise ValueError("torch inputs must be CUDA tensors (use NumPy for host memory)")
        S, Nm = stack.contiguous(), nmap.contiguous()
    ctx = ctx or _lib.context(S.device.index or 0)
    nd, R, C = S.shape
    kw = dict(method=method, semantics="evd", band_width=band_width, min_neighbors=min_neighbors,
              precision=precision, ctx=ctx)
    comps, minis = [], []
    for count, i0, i1 in ministack_plan(nd, mini_stack_size):
        # the compressed SLCs so far, then the ministack's own dates
        # (Stack.py:183-188: compressed first, order matters)
        ms = torch.cat([torch.stack(comps), S[i0:i1]]) if comps else S[i0:i1]
        out = phase_link(ms.contiguous(), Nm, half_window, mini_stack_count=count, **kw)
        minis.append(dict(count=count, start=i0, end=i1, **out))
        comps.append(out["comp"])
    comp_stack = torch.stack(comps).contiguous()
    datum = phase_link(comp_stack, Nm, half_window, mini_stack_count=1, **kw)
    res = {"ministacks": minis, "compressed": comp_stack, "datum": datum}
    if adjust:
        adj = torch.empty((nd, R, C), dtype=torch.complex64, device=S.device)
        lib = _lib.load()
        stream = torch.cuda.current_stream(S.device).cuda_stream
        for k, m in enumerate(minis):
            n_own = m["end"] - m["start"]
            own = m["phase"][-n_own:]          # the ministack's own dates
            _lib.check(lib.fpl_adjust_wrapped(ctx.handle, ctypes.c_void_p(own.data_ptr()),
                                              ctypes.c_void_p(datum["phase"][k].data_ptr()),
                                              ctypes.c_void_p(adj[m["start"]:m["end"]].data_ptr()),
                                              n_own, R * C, ctypes.c_void_p(stream)), ctx.handle)
        res["adjusted"] = adj
    if host:
        torch.cuda.synchronize(S.device)
        res = _to_numpy(res)
    return res


def _to_numpy(x):
    if isinstance(x, dict):
        return {k: _to_numpy(v) for k, v in x.items()}
    if isinstance(x, list):
        return [_to_numpy(v) for v in x]
    if _is_torch(x):
        return x.cpu().numpy()
    return x


# ---------------------------------------------------------------------------
# file level
# ---------------------------------------------------------------------------

def _raster_size(slc):
    """(width, height) of an SLC from its VRT (<slc>.vrt) or ENVI header."""
    vrt = slc + ".vrt"
    if os.path.exists(vrt):
        with open(vrt) as f:
            t = f.read()
        w = re.search(r'rasterXSize\s*=\s*"(\d+)"', t)
        h = re.search(r'rasterYSize\s*=\s*"(\d+)"', t)
        if w and h:
            return int(w.group(1)), int(h.group(1))
    for hdr in (slc + ".hdr", os.path.splitext(slc)[0] + ".hdr"):
        if os.path.exists(hdr):
            with open(hdr) as f:
                t = f.read()
            w = re.search(r"samples\s*=\s*(\d+)", t)
            h = re.search(r"lines\s*=\s*(\d+)", t)
            if w and h:
                return int(w.group(1)), int(h.group(1))
    raise FileNotFoundError("no size information (VRT or ENVI header) for " + slc)


_RAW_VRT = """<VRTDataset rasterXSize="{width}" rasterYSize="{height}">
    <VRTRasterBand dataType="CFloat32" band="1" subClass="VRTRawRasterBand">
        <sourceFilename>{path}</sourceFilename>
        <ImageOffset>0</ImageOffset>
        <PixelOffset>8</PixelOffset>
        <LineOffset>{line}</LineOffset>
        <ByteOrder>LSB</ByteOrder>
    </VRTRasterBand>
</VRTDataset>
"""

_STACK_BAND = """    <VRTRasterBand dataType="CFloat32" band="{index}">
        <SimpleSource>
            <SourceFilename>{path}</SourceFilename>
            <SourceBand>1</SourceBand>
            <SourceProperties RasterXSize="{width}" RasterYSize="{height}" DataType="CFloat32"/>
            <SrcRect xOff="{xmin}" yOff="{ymin}" xSize="{xsize}" ySize="{ysize}"/>
            <DstRect xOff="0" yOff="0" xSize="{xsize}" ySize="{ysize}"/>
        </SimpleSource>
        <Metadata domain="slc">
            <MDI key="Date">{date}</MDI>
            <MDI key="Wavelength">{wvl}</MDI>
            <MDI key="AcquisitionTime">{date}</MDI>
        </Metadata>
    </VRTRasterBand>
"""


class SlcStack:
    """A list of SLC files with their dates (Stack / MiniStack of
    src/sequential/Stack.py): the date of an SLC is the name of its folder."""

    def __init__(self, slcs, apply_bbox=None, bbox=None):
        self.slcs = list(slcs)
        self.dates = [os.path.basename(os.path.dirname(s)) for s in self.slcs]
        self.apply_bbox = list(apply_bbox) if apply_bbox is not None else [True] * len(self.slcs)
        self.bbox = bbox

    @classmethod
    def gather(cls, folder, bbox=None):
        """Stack.gatherSLCs: <folder>/*/*.slc (else *.slc.full), sorted."""
        slcs = glob.glob(os.path.join(folder, "*", "*.slc"))
        if not slcs:
            slcs = glob.glob(os.path.join(folder, "*", "*.slc.full"))
        return cls(sorted(slcs), bbox=bbox)

    def window(self, ind):
        width, height = _raster_size(self.slcs[ind])
        ymin, ymax, xmin, xmax = 0, height, 0, width
        if self.bbox and self.apply_bbox[ind]:
            ymin, ymax, xmin, xmax = self.bbox
        return width, height, xmin, ymin, xmax - xmin, ymax - ymin

    def write_vrts(self, out_dir):
        """Stack.configure + writeStackVRT: <out>/slcs/<date>.vrt per SLC and
        <out>/stack/stack.vrt over them.  Returns the stack VRT path."""
        slc_dir, stack_dir = os.path.join(out_dir, "slcs"), os.path.join(out_dir, "stack")
        os.makedirs(slc_dir, exist_ok=True)
        os.makedirs(stack_dir, exist_ok=True)
        for s, d in zip(self.slcs, self.dates):
            w, h = _raster_size(s)
            with open(os.path.join(slc_dir, d + ".vrt"), "w") as f:
                f.write(_RAW_VRT.format(width=w, height=h, path=os.path.abspath(s), line=8 * w))
        path = os.path.join(stack_dir, "stack.vrt")
        _, _, _, _, xs, ys = self.window(len(self.slcs) - 1)
        with open(path, "w") as f:
            f.write('<VRTDataset rasterXSize="{0}" rasterYSize="{1}">\n'.format(xs, ys))
            for i, d in enumerate(self.dates):
                w, h, x0, y0, xs, ys = self.window(i)
                f.write(_STACK_BAND.format(index=i + 1, path=os.path.abspath(os.path.join(slc_dir, d + ".vrt")),
                                           width=w, height=h, xmin=x0, ymin=y0, xsize=xs, ysize=ys,
                                           date=d, wvl=0.03))
            f.write("</VRTDataset>\n")
        return path


def _write_raw_vrt(slc):
    """The VRT that sequential.py:234 makes with gdal_translate -of VRT."""
    w, h = _raster_size(slc)
    with open(slc + ".vrt", "w") as f:
        f.write(_RAW_VRT.format(width=w, height=h, path=os.path.abspath(slc), line=8 * w))


def cmd_line_parser(argv=None):
    """The reference's options (src/sequential/sequential.py:9-41) plus the
    precision of the phase linking."""
    p = argparse.ArgumentParser(description="Sequential MLE phase linking over ministacks (GB300)",
                                formatter_class=argparse.ArgumentDefaultsHelpFormatter)
    p.add_argument("-i", "--inDir", dest="inputDir", required=True,
                   help="Input folder which contains folders for each SLC")
    p.add_argument("-w", "--weight_dataset", dest="weightDS", required=True, help="Input weights dataset")
    p.add_argument("-o", "--outDir", dest="outputDir", required=True, help="Output folder")
    p.add_argument("-l", "--linesperblock", type=int, dest="linesPerBlock", default=64)
    p.add_argument("-r", "--ram", type=int, dest="memorySize", default=2048, help="Memory in Mb to use")
    p.add_argument("-x", "--xhalf", type=int, dest="halfWindowX", default=29)
    p.add_argument("-y", "--yhalf", type=int, dest="halfWindowY", default=9)
    p.add_argument("-m", "--minneigh", type=int, dest="minNeighbors", default=5)
    p.add_argument("-b", "--bbox", dest="bbox", nargs="+", type=str, default=None,
                   help="bounding box: minLine maxLine minPixel maxPixel, or a VRT with a SrcRect")
    p.add_argument("-s", "--mini_stack_size", type=int, dest="miniStackSize", default=10)
    p.add_argument("-f", "--force", dest="forceprocessing", action="store_true", default=False)
    p.add_argument("--precision", default="fp32", choices=["fp32", "mixed"])
    return p.parse_args(argv)


def _bbox_from_vrt(path):
    with open(path) as f:
        t = f.read()
    m = re.search(r"<SrcRect([^>]*)/?>", t)
    if not m:
        raise ValueError("no SrcRect in " + path)
    a = dict(re.findall(r'(\w+)\s*=\s*"(-?\d+)"', m.group(1)))
    x0, y0, xs, ys = int(a["xOff"]), int(a["yOff"]), int(a["xSize"]), int(a["ySize"])
    return (y0, y0 + ys, x0, x0 + xs)


def _run_evd(inps, stack_vrt, out_dir, count, comp_dir=None, comp_name=None):
    """runEvd of sequential.py:65-99 through the Evd shim (fpl_process)."""
    from .evdlib import Evd
    aa = Evd()
    aa.inputDS = stack_vrt
    aa.weightsDS = inps.weightDS
    aa.outputFolder = out_dir
    aa.miniStackCount = count
    aa.blocksize = inps.linesPerBlock
    aa.memsize = inps.memorySize
    aa.halfWindowX = inps.halfWindowX
    aa.halfWindowY = inps.halfWindowY
    aa.minimumNeighbors = inps.minNeighbors
    aa.outputCompressedSlcFolder = comp_dir if comp_dir else out_dir
    aa.compSlc = comp_name if comp_name else "compslc.bin"
    aa.precision = inps.precision
    rc = aa.run()
    if rc:
        raise RuntimeError("phase linking of %s failed with code %d" % (stack_vrt, rc))


def run(inps):
    """The main driver of sequential.py:147-254 over files."""
    out_root = os.path.abspath(inps.outputDir)
    comp_root = os.path.join(out_root, "compressedSlc")
    os.makedirs(comp_root, exist_ok=True)
    bbox = None
    if inps.bbox is not None:
        bbox = _bbox_from_vrt(inps.bbox[0]) if os.path.isfile(inps.bbox[0]) else tuple(int(v) for v in inps.bbox)
    stack = SlcStack.gather(inps.inputDir, bbox=bbox)
    if not stack.slcs:
        raise FileNotFoundError("no SLCs under " + inps.inputDir)
    stack.write_vrts(os.path.join(out_root, "fullStack"))
    for count, i0, i1 in ministack_plan(len(stack.slcs), inps.miniStackSize):
        ms_dir = os.path.join(out_root, "miniStacks", stack.dates[i0] + "_" + stack.dates[i1 - 1])
        if os.path.isdir(ms_dir) and not inps.forceprocessing:
            print("{0} looks like it has already been processed. Skipping ... ".format(ms_dir))
            continue
        # compressed SLCs of the earlier ministacks first (Stack.py:183-188),
        # in date order, without the bounding box (they are already cut)
        comps = sorted(glob.glob(os.path.join(comp_root, "*", "*.slc")))
        mini = SlcStack(comps + stack.slcs[i0:i1], [False] * len(comps) + [True] * (i1 - i0), bbox)
        stack_vrt = mini.write_vrts(ms_dir)
        comp_dir = os.path.join(comp_root, mini.dates[-1])
        os.makedirs(comp_dir, exist_ok=True)
        comp_name = mini.dates[-1] + ".slc"
        _run_evd(inps, stack_vrt, os.path.join(ms_dir, "EVD"), count, comp_dir, comp_name)
        _write_raw_vrt(os.path.join(comp_dir, comp_name))
    # datum connection over the compressed SLCs (sequential.py:245-254)
    datum_dir = os.path.join(out_root, "Datum_connection")
    cstack = SlcStack(sorted(glob.glob(os.path.join(comp_root, "*", "*.slc"))))
    cstack.apply_bbox = [False] * len(cstack.slcs)
    stack_vrt = cstack.write_vrts(datum_dir)
    _run_evd(inps, stack_vrt, os.path.join(datum_dir, "EVD"), 1)
    return 0


def main(argv=None):
    return run(cmd_line_parser(argv))


if __name__ == "__main__":
    raise SystemExit(main())

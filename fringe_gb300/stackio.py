"""ENVI / VRT files in the layouts FRInGE's evd and phase_link modules use.

* ``write_stack``: one raw CFloat32 file per date with a per-date VRT
  (VRTRawRasterBand, as python/tops2vrt.py:143-151 writes) and a stack VRT
  whose bands carry "Date" in metadata domain "slc" (tops2vrt.py:198-216);
* ``write_nmap``: an ENVI UInt32 file, nulong bands, BIP, with HALFWINDOWX /
  HALFWINDOWY in its header (src/nmap/nmap.cpp:235-262,588-591);
* ``read_envi``: reads the module's outputs (<date>.slc, tcorr.bin,
  compressed SLC) back as arrays.
"""
import datetime
import os

import numpy as np

_ENVI_TYPES = {4: np.float32, 6: np.complex64, 13: np.uint32, 3: np.int32, 2: np.int16}


def _hdr(path, cols, rows, bands, dtype, interleave="bip", extra=None):
    lines = ["ENVI", "description = {%s}" % os.path.basename(path), "samples = %d" % cols,
             "lines = %d" % rows, "bands = %d" % bands, "header offset = 0",
             "file type = ENVI Standard", "data type = %d" % dtype,
             "interleave = %s" % interleave, "byte order = 0"]
    for k, v in (extra or {}).items():
        lines.append("%s = %s" % (k, v))
    with open(path + ".hdr", "w") as f:
        f.write("\n".join(lines) + "\n")


def dates_for(nbands, start=datetime.date(2022, 1, 1), spacing_days=12):
    return [(start + datetime.timedelta(days=spacing_days * i)).strftime("%Y%m%d") for i in range(nbands)]


def write_stack(folder, stack, dates=None):
    """Writes stack complex64 [nbands, rows, cols]; returns the stack VRT path."""
    nb, rows, cols = stack.shape
    dates = dates or dates_for(nb)
    slc_dir = os.path.join(folder, "slcs")
    os.makedirs(slc_dir, exist_ok=True)
    bands_xml = []
    for b, d in enumerate(dates):
        raw = os.path.abspath(os.path.join(slc_dir, d + ".slc.full"))
        np.ascontiguousarray(stack[b], dtype="<c8").tofile(raw)
        per_date = os.path.abspath(os.path.join(slc_dir, d + ".vrt"))
        with open(per_date, "w") as f:
            f.write('<VRTDataset rasterXSize="%d" rasterYSize="%d">\n'
                    '    <VRTRasterBand dataType="CFloat32" band="1" subClass="VRTRawRasterBand">\n'
                    '        <sourceFilename>%s</sourceFilename>\n'
                    '        <ImageOffset>0</ImageOffset>\n'
                    '        <PixelOffset>8</PixelOffset>\n'
                    '        <LineOffset>%d</LineOffset>\n'
                    '        <ByteOrder>LSB</ByteOrder>\n'
                    '    </VRTRasterBand>\n</VRTDataset>' % (cols, rows, raw, 8 * cols))
        bands_xml.append(
            '    <VRTRasterBand dataType="CFloat32" band="%d">\n'
            '        <SimpleSource>\n'
            '            <SourceFilename>%s</SourceFilename>\n'
            '            <SourceBand>1</SourceBand>\n'
            '            <SourceProperties RasterXSize="%d" RasterYSize="%d" DataType="CFloat32"/>\n'
            '            <SrcRect xOff="0" yOff="0" xSize="%d" ySize="%d"/>\n'
            '            <DstRect xOff="0" yOff="0" xSize="%d" ySize="%d"/>\n'
            '        </SimpleSource>\n'
            '        <Metadata domain="slc">\n'
            '            <MDI key="Date">%s</MDI>\n'
            '        </Metadata>\n'
            '    </VRTRasterBand>\n' % (b + 1, per_date, cols, rows, cols, rows, cols, rows, d))
    path = os.path.join(folder, "slcs_base.vrt")
    with open(path, "w") as f:
        f.write('<VRTDataset rasterXSize="%d" rasterYSize="%d">\n' % (cols, rows))
        f.write("".join(bands_xml))
        f.write("</VRTDataset>")
    return path


def write_nmap(path, nmap, ny, nx):
    """Writes nmap uint32 [rows, cols, nulong] as ENVI BIP with the window metadata."""
    rows, cols, nl = nmap.shape
    np.ascontiguousarray(nmap, dtype="<u4").tofile(path)
    _hdr(path, cols, rows, nl, 13, "bip", {"HALFWINDOWX": nx, "HALFWINDOWY": ny})
    return path


def read_envi(path):
    """Reads a single-band ENVI file written by the module (header '<path>.hdr')."""
    hdr = {}
    with open(path + ".hdr") as f:
        for line in f:
            if "=" in line:
                k, v = line.split("=", 1)
                hdr[k.strip().lower()] = v.strip()
    cols, rows, bands = int(hdr["samples"]), int(hdr["lines"]), int(hdr["bands"])
    dt = _ENVI_TYPES[int(hdr["data type"])]
    a = np.fromfile(path, dtype=np.dtype(dt).newbyteorder("<"))
    return a.reshape(rows, cols, bands)[..., 0] if bands == 1 else a.reshape(rows, cols, bands)

"""Command-line front ends with the reference's options.

``python -m fringe_gb300.cli evd ...`` mirrors src/evd/evd.py and
``python -m fringe_gb300.cli phase_link ...`` mirrors
src/phase_link/phase_link.py (same flags and defaults).
"""
import argparse
import os
import sys

from .evdlib import Evd, Phaselink


def cmd_line_parser(argv, description):
    """The options of src/evd/evd.py:6-34 (shared with phase_link.py:6-34)."""
    parser = argparse.ArgumentParser(description=description,
                                     formatter_class=argparse.ArgumentDefaultsHelpFormatter)
    parser.add_argument('-i', '--input', type=str, dest='inputDS', required=True,
                        help='Input GDAL SLC stack VRT')
    parser.add_argument('-w', '--wts', type=str, dest='wtsDS', required=True,
                        help='Input weights dataset')
    parser.add_argument('-o', '--output', type=str, dest='outputFolder', required=True,
                        help='Output folder with phase-linked SLCs')
    parser.add_argument('-l', '--linesperblock', type=int, dest='linesPerBlock', default=64,
                        help='Quantum for block of lines')
    parser.add_argument('-r', '--ram', type=int, dest='memorySize', default=2048,
                        help='Memory in Mb to use')
    parser.add_argument('-x', '--xhalf', type=int, dest='halfWindowX', default=5,
                        help='Half window size (range)')
    parser.add_argument('-y', '--yhalf', type=int, dest='halfWindowY', default=5,
                        help='Half window size (azimuth)')
    parser.add_argument('-n', '--minneigh', type=int, dest='minNeighbors', default=5,
                        help='Minimum number of neighbors for computation')
    parser.add_argument('-m', '--method', type=str, dest='method', default='MLE',
                        help='Decomposition method to use - MLE / EVD / STBAS')
    parser.add_argument('-b', '--bandwidth', type=int, dest='bandWidth', default=-1,
                        help='Diagonal bandwidth for STBAS')
    parser.add_argument('--precision', default='fp32', choices=['fp32', 'mixed'],
                        help='GPU arithmetic (fp32: plain form)')
    return parser.parse_args(argv)


def run_module(module_cls, inps):
    """runEvd of src/evd/evd.py:37-66 on this library."""
    aa = module_cls()
    aa.inputDS = inps.inputDS
    aa.weightsDS = inps.wtsDS
    aa.outputFolder = inps.outputFolder
    aa.outputCompressedSlcFolder = aa.outputFolder
    aa.compSlc = "compslc.bin"
    aa.blocksize = inps.linesPerBlock
    aa.memsize = inps.memorySize
    aa.halfWindowX = inps.halfWindowX
    aa.halfWindowY = inps.halfWindowY
    aa.minimumNeighbors = inps.minNeighbors
    aa.method = inps.method
    aa.bandWidth = inps.bandWidth
    aa.precision = inps.precision
    return aa.run()


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv or argv[0] not in ("evd", "phase_link"):
        print("usage: python -m fringe_gb300.cli {evd,phase_link} [options]")
        return 2
    which = argv.pop(0)
    inps = cmd_line_parser(argv, 'Perform MLE-based phase-linking on a stack of coregistered SLCs')
    return run_module(Evd if which == "evd" else Phaselink, inps)


if __name__ == "__main__":
    sys.exit(main())

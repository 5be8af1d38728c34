"""Command line, as zorro's (zorro/__main__.py:13-107):

    python -m zorro_gb300 -c movie.zor [-i movie.mrcs] [-o sum.mrc]

* no ``-c`` and no ``-i``: writes ``template.zor`` (the default settings) and
  exits;
* ``-c`` alone: loads the config and the movie it names (``files['stack']``);
* ``-c`` and ``-i``: loads the config, then the given movie;
* ``-o``: the name of the aligned sum.

Then the movie is registered on the GPU (triMode 'refine' first registers
with 'diag' unless the config already holds a registration), the sums are
saved (``saveData``), and the config is written back with METAstatus
'fini'.  Diagnostic plots (``savePNG``) are not drawn.
"""
from __future__ import annotations

import sys
import time


def parse(argv):
    opts = {"-c": None, "-i": None, "-o": None}
    it = iter(range(len(argv)))
    for j in it:
        if argv[j] in opts and j + 1 < len(argv):
            opts[argv[j]] = argv[j + 1]
            next(it, None)
    return opts["-c"], opts["-i"], opts["-o"]


def main(argv=None):
    from .registrator import ImageRegistrator
    argv = sys.argv[1:] if argv is None else argv
    config, infile, outfile = parse(argv)
    reg = ImageRegistrator()
    if infile is None and config is None:
        print("No input files, outputing template.zor")
        reg.saveConfig(configNameIn="template.zor")
        return 0
    if config is not None:
        reg.loadConfig(configNameIn=config, loadData=infile is None)
    reg.bench["total0"] = time.time()
    if infile is not None:
        reg.files["stack"] = infile
        reg.loadData()
    if reg.images is None:
        raise ValueError("zorro_gb300: the config names no movie (files['stack']) and no -i was given")
    if outfile is not None:
        reg.files["sum"] = outfile
    if reg.triMode == "refine":
        if reg.errorDictList and reg.imageSum is not None:
            print("Zorro refine assuming that initial alignment has already been performed.")
        else:
            print("Zorro refine performing initial alignment.")
            reg.triMode = "diag"
            reg.alignImageStack()
            reg.loadData()  # the shifted frames are replaced by the raw movie again
        reg.triMode = "refine"
    reg.alignImageStack()
    reg.saveData()
    reg.bench["total1"] = time.time()
    reg.METAstatus = "fini"
    reg.saveConfig()
    print("Zorro exiting")
    return 0


if __name__ == "__main__":
    sys.exit(main())

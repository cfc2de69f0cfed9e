"""Image ingest as the CLI picks it (cli/src/main.rs:129-137,
cli/src/image/mod.rs): by the file extension, "jpg"/"jpeg" -> JPEG,
"png" -> PNG, anything else is refused.  Both return (width, height, RGBA8
array (h, w, 4))."""
import os

from . import jpegio, pngio


def read_image(path):
    ext = os.path.splitext(str(path))[1].lower().lstrip(".")
    if not ext:
        raise ValueError("input filename has no extension, can't guess type")
    if ext in ("jpg", "jpeg"):
        return jpegio.read_jpeg(path)
    if ext == "png":
        return pngio.read_png(path)
    raise ValueError("unsupported input file type: %s" % ext)

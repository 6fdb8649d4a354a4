"""Species headers compiled into the step kernels at run time.

The reference compiles its OpenCL kernels at start-up with the species header
named on its command line (src/abms.c:565-568); its shipped properties.h is
built into this library. ``Species(path)`` compiles the step kernels with
NVRTC against another properties.h-style header (sampo_species_compile) for
one GPU; simulations and batches use it after ``set_species``."""
from __future__ import annotations

import ctypes as C

from . import _lib
from ._lib import SampoError

LOG_BYTES = 1 << 16


class Species:
    def __init__(self, header_path: str | None = None, text: str | None = None, device: int = 0, name: str = "species.h"):
        if (header_path is None) == (text is None):
            raise ValueError("give a header path or its text")
        self.lib = _lib.load()
        h = C.c_void_p()
        log = C.create_string_buffer(LOG_BYTES)
        if header_path is not None:
            rc = self.lib.sampo_species_compile(header_path.encode(), device, log, LOG_BYTES, C.byref(h))
        else:
            rc = self.lib.sampo_species_compile_text(name.encode(), text.encode(), device, log, LOG_BYTES, C.byref(h))
        self.log = log.value.decode(errors="replace")
        if rc != 0:
            raise SampoError(rc, self.log)
        self.h = h

    @staticmethod
    def check(text: str, sm: int = 103, name: str = "species.h") -> tuple[int, str]:
        """Compile without loading (no GPU needed): (status, compiler log)."""
        lib = _lib.load()
        log = C.create_string_buffer(LOG_BYTES)
        rc = lib.sampo_species_check_text(name.encode(), text.encode(), sm, log, LOG_BYTES)
        return rc, log.value.decode(errors="replace")

    def close(self):
        if getattr(self, "h", None):
            self.lib.sampo_species_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

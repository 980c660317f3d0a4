"""ctypes declarations of the batched, MC3 and serving entry points."""


def declare_ext(lib):
    return lib

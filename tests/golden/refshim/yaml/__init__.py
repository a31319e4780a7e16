def safe_load(stream):
    raise RuntimeError("yaml is unavailable in the fixture shim")


load = safe_load

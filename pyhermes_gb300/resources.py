"""Catalogue path resolution (pyhermes/io/resources.py): HTTP(S) detection,
SHA256 checks of local files, and the deterministic cache location of a
downloaded catalogue.  A cached copy of a remote catalogue is reused (after
its checksum, when one is given); fetching a missing one needs the network,
which this package does not use, so that case raises with the cache path
to place the file at."""
import hashlib
import logging
import os
from pathlib import Path
from urllib.parse import unquote, urlparse

logger = logging.getLogger(__name__)

_REMOTE_SCHEMES = {"http", "https"}
_CHUNK = 1024 * 1024


def is_remote_url(path):
    """resources.py:28-32: whether ``path`` is an http(s) URL."""
    if not isinstance(path, (str, os.PathLike)):
        return False
    return urlparse(os.fspath(path)).scheme.lower() in _REMOTE_SCHEMES


def file_sha256(path, chunk_size=_CHUNK):
    """resources.py:35-41: hexadecimal SHA256 of a local file."""
    digest = hashlib.sha256()
    with Path(path).open("rb") as f:
        for chunk in iter(lambda: f.read(chunk_size), b""):
            digest.update(chunk)
    return digest.hexdigest()


def _normalize_sha256(value):
    """resources.py:44-52: None, or 64 lowercase hex digits ('sha256:' prefix allowed)."""
    if value in (None, ""):
        return None
    value = str(value).lower()
    if value.startswith("sha256:"):
        value = value.split(":", 1)[1]
    if len(value) != 64 or any(c not in "0123456789abcdef" for c in value):
        raise ValueError("sha256 must be a 64-character hexadecimal digest.")
    return value


def _default_cache_dir():
    """resources.py:55-62: $PYHERMES_CACHE_DIR, $XDG_CACHE_HOME/pyhermes, ~/.cache/pyhermes."""
    configured = os.environ.get("PYHERMES_CACHE_DIR")
    if configured:
        return Path(configured).expanduser()
    xdg = os.environ.get("XDG_CACHE_HOME")
    if xdg:
        return Path(xdg).expanduser() / "pyhermes"
    return Path.home() / ".cache" / "pyhermes"


def remote_cache_path(url, cache_dir=None):
    """resources.py:65-74: <cache>/<first 12 hex of sha256(url)>-<file name>."""
    root = Path(cache_dir).expanduser() if cache_dir else _default_cache_dir()
    name = Path(unquote(urlparse(str(url)).path)).name or "download"
    return root / f"{hashlib.sha256(str(url).encode('utf-8')).hexdigest()[:12]}-{name}"


def _verify_checksum(path, expected, source):
    if expected is None:
        return
    actual = file_sha256(path)
    if actual != expected:
        raise ValueError(f"SHA256 mismatch for {source}: expected {expected}, got {actual}.")


def resolve_data_path(path, *, cache_path=None, cache_dir=None, sha256=None, timeout=60):
    """resources.py:87-160: a local path (checksum-verified when sha256 is
    given) or the cached copy of an http(s) catalogue."""
    source = os.fspath(path)
    expected = _normalize_sha256(sha256)
    if not is_remote_url(source):
        local = Path(source).expanduser()
        _verify_checksum(local, expected, str(local))
        return str(local)
    if cache_path and cache_dir:
        raise ValueError("Set only one of cache_path and cache_dir.")
    target = Path(cache_path).expanduser() if cache_path else remote_cache_path(source, cache_dir=cache_dir)
    if target.is_file():
        try:
            _verify_checksum(target, expected, str(target))
        except ValueError:
            logger.warning("Cached file failed checksum verification: %s", target)
        else:
            logger.info("Using cached particle data: %s", target)
            return str(target)
    raise ValueError(f"Remote catalogue '{source}' is not in the cache and fetching it needs network access; "
                     f"place the file at {target} (or pass the local path).")

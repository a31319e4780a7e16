"""JSON with // comments, enough for the reference's default_params.json."""
import json as _json
import re as _re


def loads(text, *args, **kwargs):
    text = _re.sub(r"(?m)^\s*//[^\n]*$", "", text)
    text = _re.sub(r"([,{\[\]\"0-9el])\s*//[^\n]*", r"\1", text)
    text = _re.sub(r",(\s*[}\]])", r"\1", text)
    return _json.loads(text)


def load(fp, *args, **kwargs):
    return loads(fp.read())

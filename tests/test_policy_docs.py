"""Every policy key that vta_ctx_set_policy accepts is documented for the
maintainer (the binding guide lists each key with its values)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_policy_key_is_documented():
    src = open(os.path.join(ROOT, "vectorta_gb300", "csrc", "vta_api.cu")).read()
    body = src[src.index("vta_status vta_ctx_set_policy("):]
    body = body[: body.index("unknown policy key")]
    keys = sorted(set(re.findall(r'k == "([a-z_]+)"', body)))
    assert len(keys) >= 8, keys
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [k for k in keys if f'"{k}"' not in guide]
    assert not missing, missing

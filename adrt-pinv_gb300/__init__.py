"""GB300-native explicit oblique inverses of the ADRT (drop-in for dsrim/adrt-pinv's fastops/fastcpp path)."""

from . import phantoms  # noqa: F401

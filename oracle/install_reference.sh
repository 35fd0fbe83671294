#!/usr/bin/env bash
# Installs the reference package (gstenzel/qandle 0.1.8, pure Python on torch)
# into baseline/_ref, where bench.py's CPU baselines import it.  Test and
# benchmark infrastructure only; baseline/_ref is git-ignored.
#
# The reference builds with poetry-core, which is not in the offline
# wheelhouse, so pip cannot run its declared build backend.  The package is
# pure Python: the source tree is copied to /tmp, its [build-system] table is
# replaced by a setuptools one that packages the same src/qandle tree, and
# that copy is pip-installed with --no-deps.  The package's code is not
# changed.  Its dependency qw_map (qw-map 0.1.2) is not installed either;
# bench.py supplies a stand-in for `qw_map.none` (identity) at import time.
set -euo pipefail
SRC=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
DEST=$(cd "$HERE/.." && pwd)/baseline/_ref
TMP=$(mktemp -d /tmp/qandle_ref.XXXXXX)
cp -r "$SRC/src" "$SRC/README.md" "$SRC/LICENSE" "$TMP/"
cat > "$TMP/pyproject.toml" <<'EOF'
[build-system]
requires = ["setuptools"]
build-backend = "setuptools.build_meta"

[project]
name = "qandle"
version = "0.1.8"

[tool.setuptools.packages.find]
where = ["src"]
exclude = ["qandle.test*"]
EOF
rm -rf "$DEST"
python -m pip install --no-index --no-build-isolation --no-deps --find-links /opt/wheelhouse \
    --target "$DEST" "$TMP" >"$TMP/pip.log" 2>&1 || { tail -20 "$TMP/pip.log"; exit 1; }
rm -rf "$TMP"
echo "installed into $DEST"

"""qandle_gb300 (package init is written below)."""

"""Monitors and detectors (acc/components/monitors)."""

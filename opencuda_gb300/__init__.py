"""GB300-native HoughLine (drop-in for OpenCUDA HoughLine)."""

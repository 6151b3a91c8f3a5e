"""GB300-native zfp block codec."""

"""GB300-native direct-optimization scoring path of POY/poyd."""

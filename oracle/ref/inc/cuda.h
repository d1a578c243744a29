/* empty stand-in: see cuda_runtime_api.h */

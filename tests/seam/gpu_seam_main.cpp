// The `--gpu` link seam: raw_native_cli's GPU branch (app/main.cpp:321-330) over the
// reference's own parser and src/tools/gpu_run.cpp, with raw::gpuInit / raw::renderGpu
// resolved to the CUDA shim (gpu_shim.cpp over librn_ao.so) and the AO passes to the AO shim.
// `--gpu` is implied; the other flags are the CLI's. Exit codes are gpu_run.cpp's: 0 after
// both frames and the GPU certificate, 2 on bad input or unwritable output, 4 without a GPU
// ("unverifiable", with the reason in gpu_certificate.json).
#include "raw/renderer/gpu.hpp"
#include "raw/tools/cli_params.hpp"
#include "raw/tools/gpu_run.hpp"
#include <cstdio>
#include <string>
#include <vector>

int main(int argc, char** argv) {
    std::vector<const char*> args(argv, argv + argc);
    args.push_back("--gpu");
    std::string err;
    std::optional<raw::CliParams> parsed = raw::parseArgs((int)args.size(), args.data(), err);
    if (!parsed) { std::printf("param error: %s\n", err.c_str()); return 2; }
    raw::CliParams p = *parsed;
    p.gpuBackend = raw::gpuBackendName();
    return raw::runGpu(p);
}

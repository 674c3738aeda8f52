// mcd_gpu_cli.cpp -- the reference's JSON CLI (apps/mcd_cli/main.cpp) on the GPU
// engine: one flat JSON request object on stdin, one object on stdout; exit code
// 0, or {"error": message} and exit code 1.  The request handling lives in the
// shim library (request.cpp, CLI dialect), shared with the Lambda-style handler.
#include <cstdio>
#include <iostream>
#include <iterator>
#include <string>

#include "mcd_shim.hpp"

int main() {
    const std::string input((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
    int status = MCD_SHIM_INTERNAL_ERROR;
    char* out = mcd_shim_handle_request(input.c_str(), MCD_SHIM_DIALECT_CLI, 0, &status);
    if (!out) {
        std::cout << "{\"error\":\"out of memory\"}\n";
        return 1;
    }
    std::cout << out << "\n";
    mcd_shim_free(out);
    return status == MCD_SHIM_OK ? 0 : 1;
}

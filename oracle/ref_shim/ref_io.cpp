// File-path shim of the reference build (test infrastructure).
//
// The reference's main() reads and writes fixed absolute paths under
// /home/davidxu/ (main.cu:3251-3252).  oracle/ref_cuda.sh links the reference
// build with -Wl,--wrap=fopen, so each fopen() of the program lands here: a path
// under /home/davidxu/ is opened inside the directory named by $PRGPU_REF_IO_DIR
// instead, any other path as given.  The reference files themselves are not
// changed.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

extern "C" FILE* __real_fopen(const char* path, const char* mode);

extern "C" FILE* __wrap_fopen(const char* path, const char* mode) {
    static const char prefix[] = "/home/davidxu/";
    const char* dir = getenv("PRGPU_REF_IO_DIR");
    if (dir && path && strncmp(path, prefix, sizeof prefix - 1) == 0) {
        std::string p = std::string(dir) + "/" + (path + sizeof prefix - 1);
        return __real_fopen(p.c_str(), mode);
    }
    return __real_fopen(path, mode);
}

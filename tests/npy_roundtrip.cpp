// Test helper: read an .npy file with the library's reader and write it back as float64.
#include <cstdio>
#include "npy.h"
int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    try {
        npy::Array a = npy::read(argv[1]);
        std::vector<double> v = npy::as_double(a);
        npy::write(argv[2], v.data(), a.shape);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}

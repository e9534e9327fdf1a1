// Test infrastructure: drives the reference's own multiscaler programs
// (multiscaler/decompose.cpp, recompose.cpp, merge_coarse.cpp, built with
// their main renamed, over multiscaler/multiscaler.cpp) on in-memory
// images.  The two iio entry points that multiscaler.cpp calls
// (read_image / save_image, multiscaler/multiscaler.cpp:115-127) are
// supplied here over a table of named images instead of files, so a test
// stores its input under a name, runs a program with the same command line
// as the multiscale script (src/utils/VBM3Ddenoising_multiscale.sh), and
// reads the outputs back by name.  Images are interleaved rows x columns x
// channels floats, as iio hands them to multiscaler::Image.
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {
struct Stored {
    int w, h, c;
    std::vector<float> v;
};
std::map<std::string, Stored>& table()
{
    static std::map<std::string, Stored> t;
    return t;
}
}  // namespace

// the programs' renamed mains (C++ linkage, as main had)
int ms_decompose_main(int argc, char* argv[]);
int ms_recompose_main(int argc, char* argv[]);
int ms_merge_coarse_main(int argc, char* argv[]);

extern "C" {

float* iio_read_image_float_vec(const char* fname, int* w, int* h, int* pd)
{
    auto it = table().find(fname);
    if (it == table().end()) return nullptr;
    const Stored& s = it->second;
    float* p = (float*)std::malloc(sizeof(float) * s.v.size());
    std::memcpy(p, s.v.data(), sizeof(float) * s.v.size());
    *w = s.w;
    *h = s.h;
    *pd = s.c;
    return p;
}

void iio_save_image_float_vec(char* filename, float* x, int w, int h, int pd)
{
    Stored s{w, h, pd, std::vector<float>(x, x + (size_t)w * h * pd)};
    table()[filename] = std::move(s);
}

// Stores an image (w x h x c, interleaved) under `name`.
void msref_put(const char* name, const float* data, int w, int h, int c)
{
    iio_save_image_float_vec(const_cast<char*>(name), const_cast<float*>(data), w, h, c);
}

// Size of a stored image (0 if absent), and its pixels when out != NULL.
int msref_get(const char* name, float* out, int* w, int* h, int* c)
{
    auto it = table().find(name);
    if (it == table().end()) return 0;
    const Stored& s = it->second;
    *w = s.w;
    *h = s.h;
    *c = s.c;
    if (out) std::memcpy(out, s.v.data(), sizeof(float) * s.v.size());
    return 1;
}

void msref_clear(void) { table().clear(); }

// Runs one program with argv[0..argc) (argv[0] is the program name).
int msref_run(const char* program, int argc, char** argv)
{
    std::vector<char*> a(argv, argv + argc);
    a.push_back(nullptr);
    if (!std::strcmp(program, "decompose")) return ms_decompose_main(argc, a.data());
    if (!std::strcmp(program, "recompose")) return ms_recompose_main(argc, a.data());
    if (!std::strcmp(program, "merge_coarse")) return ms_merge_coarse_main(argc, a.data());
    return -1;
}

}  // extern "C"

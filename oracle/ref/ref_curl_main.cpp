// Driver for the reference curl generator (ImageUtils.cpp).
//   ref_curlgen OUT.tga     runs GenerateCurlNoise (ImageUtils.cpp:176) and writes its TGA;
//   ref_curlgen --hash      prints hashNoise(x, y, z) (ImageUtils.cpp:25) for each "x y z" on stdin.
#include <cstdio>
#include <cstring>
#include <string>
void GenerateCurlNoise(std::string path);
float hashNoise(float x, float y, float z);
int main(int argc, char** argv) {
    if (argc < 2) return 2;
    if (strcmp(argv[1], "--hash") == 0) {
        float x, y, z;
        while (scanf("%f %f %f", &x, &y, &z) == 3) printf("%.9g %.9g %.9g %.9g\n", x, y, z, hashNoise(x, y, z));
        return 0;
    }
    GenerateCurlNoise(argv[1]);
    return 0;
}

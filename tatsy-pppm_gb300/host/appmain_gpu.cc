// GPU counterpart of the reference driver (main/appmain.cc:11-26): the same
// main(width, height, spp) flow through the host mirror, with the scene
// given on the command line because the reference's contest assets are not
// all available:
//
//   appmain_gpu <width> <height> <spp> <mesh.ply> <env.hdr> <out.ppm> [photons] [compat|canonical|pt]
//               [result directory: per-pass PNG files as the reference writes them]
//
// The mesh gets a Lambertian material on a checker floor of mirror and
// Phong tiles like appmain.cc:97-112. The result is written after the last
// pass exactly as the reference prepares its PNG (flip rows, divide by the
// pass count, gamma 1/2.2, clamp, x255; ppm_probabilistic.cc:97-106,
// image.cc:202-213,530-532) but as a binary PPM.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "pppm.hpp"

int main(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s width height spp mesh.ply env.hdr out.ppm [photons] [compat|canonical|pt] [dir]\n",
                     argv[0]);
        return 2;
    }
    const int width = std::atoi(argv[1]);
    const int height = std::atoi(argv[2]);
    const int spp = std::atoi(argv[3]);
    const int photons = argc >= 8 ? std::atoi(argv[7]) : 200000;
    const std::string mode = argc >= 9 ? argv[8] : "compat";
    try {
        Scene scene;
        Trimesh mesh(argv[4]);
        scene.add(mesh, LambertianBRDF::factory(Vector3D(0.75, 0.75, 0.75)));
        const int tiles = 8;
        const double tile = 8.0;
        for (int i = 0; i < tiles; i++)
            for (int j = 0; j < tiles; j++) {
                const double ii = (i - tiles / 2) * tile, jj = (j - tiles / 2) * tile;
                const Vector3D p00(ii, -10.0, jj), p01(ii + tile, -10.0, jj), p10(ii, -10.0, jj + tile),
                    p11(ii + tile, -10.0, jj + tile);
                const bool even = (i + j) % 2 == 0;
                const BSDF b = even ? PhongBRDF::factory(Vector3D(0.9, 0.9, 0.9), 128.0)
                                    : SpecularBRDF::factory(Vector3D(0.2, 0.2, 0.2));
                scene.add(Triangle(p00, p11, p01), b);
                scene.add(Triangle(p00, p10, p11), b);
            }
        scene.setEnvmap(Envmap(argv[5]));
        scene.setAccelerator();
        const Vector3D eye(-25.0, 5.0, -18.0);
        Camera camera(eye, -eye.normalized(), Vector3D(0.0, 1.0, 0.0), 0.9, width, height, 1.0);
        RenderParameters params(photons, spp, 128, 16.0);
        const std::string dir = argc >= 10 ? argv[9] : "";
        std::vector<float> img;
        if (mode == "pt") {
            PathTracing pt;
            pt.resultDirectory = dir;
            pt.render(scene, camera, params);
            img = pt.result();
        } else {
            ProgressivePhotonMappingProb ppm;
            ppm.mode = mode == "canonical" ? PPPM_MODE_CANONICAL : PPPM_MODE_COMPAT;
            ppm.resultDirectory = dir;
            ppm.render(scene, camera, params);
            img = ppm.result();
        }
        FILE* f = std::fopen(argv[6], "wb");
        if (!f) throw pppm::Error(PPPM_E_ARG, std::string("cannot write ") + argv[6]);
        std::fprintf(f, "P6\n%d %d\n255\n", width, height);
        for (int y = height - 1; y >= 0; y--)
            for (int x = 0; x < width; x++)
                for (int c = 0; c < 3; c++) {
                    double v = std::pow((double)img[3 * ((size_t)y * width + x) + c], 1.0 / 2.2);
                    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
                    std::fputc((int)(unsigned char)(255.0 * v), f);
                }
        std::fclose(f);
        std::printf("rendered %dx%d, %d passes, %zu triangles\n", width, height, spp, scene.numTriangles());
    } catch (const pppm::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}

// Headless driver for the reference's 2D voxel canvas (Canvas2D_CC.cpp),
// compiled against the reference's own source (see oracle/build_ref.sh).
// Test infrastructure only: it produces the golden voxel masks that pin the
// canvas restatement (oracle/canvas_oracle.py) and the GPU canvas.
//
// usage: ref_canvas <ops.txt> <out.bin>
//   ops.txt   first line "canvas <width> <height> <offset>", then one
//             operation per line, applied in order:
//               circle <cx> <cy> <r>
//               ring <cx> <cy> <r_outer> <r_inner>
//               rect <cx> <cy> <sx> <sy> <rotation>
//               prism <cx> <cy> <sx> <sy> <extra> <rotation>
//               cutcircle <cx> <cy> <r>
//               cutrect <cx> <cy> <sx> <sy> <rotation>
//   out.bin   uint32 nx, uint32 ny, then one byte per voxel in voxel order
//             (x fastest): bit 0 active, bit 1 surface.
#include "Canvas2D_CC.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s ops.txt out.bin\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[1]);
    std::string line;
    Canvas2D_CC* canvas = nullptr;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string op;
        if (!(ss >> op)) continue;
        double a[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 6 && (ss >> a[k]); ++k) {
        }
        if (op == "canvas") {
            canvas = new Canvas2D_CC(glm::dvec2(a[0], a[1]), a[2]);
            continue;
        }
        if (!canvas) return 3;
        const glm::dvec2 c(a[0], a[1]);
        if (op == "circle")
            canvas->drawCircle(c, a[2]);
        else if (op == "ring")
            canvas->drawRing(c, a[2], a[3]);
        else if (op == "rect")
            canvas->drawRectangle(c, glm::dvec2(a[2], a[3]), a[4]);
        else if (op == "prism")
            canvas->drawPrism(c, glm::dvec2(a[2], a[3]), a[4], a[5]);
        else if (op == "cutcircle")
            canvas->cutCircle(c, a[2]);
        else if (op == "cutrect")
            canvas->cutRectangle(c, glm::dvec2(a[2], a[3]), a[4]);
        else
            return 4;
    }
    if (!canvas) return 3;
    FILE* f = fopen(argv[2], "wb");
    if (!f) return 5;
    const uint32_t nx = canvas->u2_Size.x, ny = canvas->u2_Size.y;
    fwrite(&nx, 4, 1, f);
    fwrite(&ny, 4, 1, f);
    for (size_t i = 0; i < canvas->v_Voxels.size(); ++i) {
        const Voxel_ST* v = canvas->v_Voxels[i];
        const uint8_t b = (uint8_t)((v->b_Active ? 1 : 0) | (v->b_Surface ? 2 : 0));
        fwrite(&b, 1, 1, f);
    }
    fclose(f);
    delete canvas;
    return 0;
}

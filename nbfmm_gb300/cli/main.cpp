// main.cpp -- nbfmm_main: the reference's movie program (main/main.cu) on the GB300 engine.
//
// Same command line, same checks, same printed lines and the same .y4m output as main/main.cu:25-262:
//   nbfmm_main <output file> <width> <height> <fps> <time (second)> <FMM level> <number of stars>
//              <position width> <position height> <display scale> <grav_const> <size_scale> <model> [parameters]
// with the models circle, circle-uniform, disk, disk-center, disk-static, double-disk, double-disk-center and
// rectangle. Usage errors print the reference's usage line and abort(), as the reference does. The frames come
// from the engine (Stars update, display, prune) through the C ABI; the file write of a frame overlaps the
// GPU work of the next one.
//
// Reference behaviour kept: the tick is 0.05 / fps (main.cu:52); double-disk centres are placed along the
// display diagonal by the proportions (main.cu:163-166); double-disk-center passes its first centre weight for
// both disks (main.cu:204). Changed: double-disk-center requires its eccentricity argument (the reference reads
// argv[21] after checking only argc > 20, main.cu:175-190); a failed engine call prints its message and aborts
// where the reference would carry on unchecked; stars beyond num_star * p1 + num_star * p2 of a double disk are
// zero (the reference leaves that device memory uninitialised).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "nbfmm_gb300.h"

using namespace std;

namespace {

void check(int rc, const char* what) {
  if (rc != NBFMM_OK) {
    fflush(stdout);
    fprintf(stderr, "%s: %s\n", what, nbfmm_last_error());
    abort();
  }
}

void require(bool ok, const char* what) {
  if (!ok) {
    fflush(stdout);
    fprintf(stderr, "nbfmm_main: %s\n", what);
    abort();
  }
}

struct F2 {
  float x, y;
};

}  // namespace

int main(int argc, char const* argv[]) {
  cout << "NBFMM " << 1 << "." << 2 << "." << 0 << endl << endl;  // the interface version mirrored

  if (argc <= 13) {
    cout << "Usage: " << argv[0]
         << " <output file> <width> <height> <fps> <time (second)>"
            " <FMM level> <number of stars> <position width> <position height> <display scale> <grav_const>"
            " <size_scale> <model> [model parameters] ..."
         << endl << endl;
    abort();
  }

  const char* result_y4m = argv[1];
  const int width = atoi(argv[2]);
  const int height = atoi(argv[3]);
  const int fps = atoi(argv[4]);
  const int num_second = atoi(argv[5]);
  const int num_frame = num_second * fps;
  const int fmm_level = atoi(argv[6]);
  const int num_star = atoi(argv[7]);
  const float pos_width = atof(argv[8]);
  const float pos_height = atof(argv[9]);
  const float display_scale = atof(argv[10]);
  const float tick = 0.05 / fps;
  const float grav_const = atof(argv[11]);
  const float size_scale = atof(argv[12]);

  const float position_limits[4] = {-pos_width / 2, -pos_height / 2, pos_width / 2, pos_height / 2};
  const float display_limits[4] = {position_limits[0] * display_scale, position_limits[1] * display_scale,
                                   position_limits[2] * display_scale, position_limits[3] * display_scale};
  const float center_position[2] = {0.0f, 0.0f};
  const char* model = argv[13];

  printf("%d x %d pixel, %d fps, %d sec / %d frame\n", width, height, fps, num_second, num_frame);
  printf("%d FMM level, %d stars, tick = %.6f, grav const = %.2f, scale size = %.2f\n", fmm_level, num_star, tick,
         grav_const, size_scale);
  printf("position size = %.2f x %.2f, display scale = %.2f\n", pos_width, pos_height, display_scale);
  printf("position range = [%.2f, %.2f] x [%.2f, %.2f], display range = [%.2f, %.2f] x [%.2f, %.2f]\n",
         position_limits[0], position_limits[2], position_limits[1], position_limits[3], display_limits[0],
         display_limits[2], display_limits[1], display_limits[3]);
  printf("\n");

  // Stars::Stars (stars.cu:15-50) and its asserts.
  require(width > 0 && height > 0 && fps > 0 && size_scale > 0, "width, height, fps and size_scale must be > 0");
  require(display_limits[0] < display_limits[2] && display_limits[1] < display_limits[3],
          "display limits must be ordered");
  nbfmm_stars* stars = nullptr;
  check(nbfmm_stars_create(fmm_level, num_star, tick, grav_const, position_limits, &stars), "Stars");
  const float tick_ = tick * std::sqrt(grav_const);  // stars.cu:31, the tick the models receive
  float *cur = nullptr, *prev = nullptr, *w = nullptr;
  check(nbfmm_stars_state(stars, &cur, &prev, &w), "Stars");

  if (!strcmp(model, "circle")) {
    if (argc <= 16) {
      cout << "Usage: " << argv[0] << " ... circle <radius> <weight> <center weight>" << endl << endl;
      abort();
    }
    const float radius = atof(argv[14]);
    const float weight = atof(argv[15]);
    const float weight_center = atof(argv[16]);
    printf("Model Circle: radius = %.2f, weight = %.2f, center weight = %.2f\n\n", radius, weight, weight_center);
    check(nbfmm_model_circle_center(num_star, center_position, radius, weight, weight_center, tick_, cur, prev, w,
                                    nullptr),
          "generateCircleCenter");
  } else if (!strcmp(model, "circle-uniform")) {
    if (argc <= 16) {
      cout << "Usage: " << argv[0] << " ... circle-uniform <radius> <weight> <center weight>" << endl << endl;
      abort();
    }
    const float radius = atof(argv[14]);
    const float weight = atof(argv[15]);
    const float weight_center = atof(argv[16]);
    printf("Model Uniform Circle: radius = %.2f, weight = %.2f, center weight = %.2f\n\n", radius, weight,
           weight_center);
    check(nbfmm_model_circle_uniform_center(num_star, center_position, radius, weight, weight_center, tick_, cur,
                                            prev, w, nullptr),
          "generateCircleUniformCenter");
  } else if (!strcmp(model, "disk")) {
    if (argc <= 15) {
      cout << "Usage: " << argv[0] << " ... disk <radius> <weight>" << endl << endl;
      abort();
    }
    const float radius = atof(argv[14]);
    const float weight = atof(argv[15]);
    printf("Model Disk: radius = %.2f, weight = %.2f\n\n", radius, weight);
    check(nbfmm_model_disk(num_star, center_position, radius, weight, tick_, cur, prev, w, nullptr), "generateDisk");
  } else if (!strcmp(model, "disk-center")) {
    if (argc <= 16) {
      cout << "Usage: " << argv[0] << " ... disk-center <radius> <weight> <center weight>" << endl << endl;
      abort();
    }
    const float radius = atof(argv[14]);
    const float weight = atof(argv[15]);
    const float weight_center = atof(argv[16]);
    printf("Model Centered Disk: radius = %.2f, weight = %.2f, center weight = %.2f\n\n", radius, weight,
           weight_center);
    check(nbfmm_model_disk_center(num_star, center_position, radius, weight, weight_center, tick_, cur, prev, w,
                                  nullptr),
          "generateDiskCenter");
  } else if (!strcmp(model, "disk-static")) {
    if (argc <= 15) {
      cout << "Usage: " << argv[0] << " ... disk-static <radius> <weight>" << endl << endl;
      abort();
    }
    const float radius = atof(argv[14]);
    const float weight = atof(argv[15]);
    printf("Model Centered Disk: radius = %.2f, weight = %.2f\n\n", radius, weight);  // the reference's label
    check(nbfmm_model_disk_static(num_star, center_position, radius, weight, tick_, cur, prev, w, nullptr),
          "generateDiskStatic");
  } else if (!strcmp(model, "double-disk") || !strcmp(model, "double-disk-center")) {
    const bool centered = !strcmp(model, "double-disk-center");
    if (argc <= (centered ? 21 : 19)) {
      if (centered) {
        cout << "Usage: " << argv[0]
             << " ... double-disk-center <proportion 1> <proportion 2> <radius 1> <radius 2>"
                " <weight> <center weight> <eccentricity>"
             << endl << endl;
      } else {
        cout << "Usage: " << argv[0]
             << " ... double-disk <proportion 1> <proportion 2> <radius 1> <radius 2> <weight> <eccentricity>"
             << endl << endl;
      }
      abort();
    }
    const float n1 = atof(argv[14]);
    const float n2 = atof(argv[15]);
    const float p1 = n1 / (n1 + n2);
    const float p2 = n2 / (n1 + n2);
    const float radius1 = atof(argv[16]);
    const float radius2 = atof(argv[17]);
    const float weight = atof(argv[18]);
    const float weight_center1 = centered ? (float)atof(argv[19]) : 0.0f;
    const float eccentricity = atof(argv[centered ? 21 : 19]);
    require(n1 >= 0 && n2 >= 0, "proportions must be >= 0");
    // main.cu:163-166: (lower-left * p1 + upper-right * (p1 + 2 p2)) / 2 and its mirror.
    const float a1 = 1 * p1 + 0 * p2, b1 = 1 * p1 + 2 * p2;
    const float a2 = 1 * p2 + 0 * p1, b2 = 1 * p2 + 2 * p1;
    const F2 c1 = {(display_limits[0] * a1 + display_limits[2] * b1) / 2,
                   (display_limits[1] * a1 + display_limits[3] * b1) / 2};
    const F2 c2 = {(display_limits[2] * a2 + display_limits[0] * b2) / 2,
                   (display_limits[3] * a2 + display_limits[1] * b2) / 2};
    const float center1[2] = {c1.x, c1.y}, center2[2] = {c2.x, c2.y};
    printf("Model Double Disk: proportion = %.2f / %.2f, radius = %.2f / %.2f, weight = %.2f, eccentricity = %.2f\n\n",
           n1, n2, radius1, radius2, weight, eccentricity);
    const int k1 = (int)(num_star * p1), k2 = (int)(num_star * p2);
    if (centered) {
      check(nbfmm_model_double_disk_center(k1, k2, center1, center2, radius1, radius2, weight, weight_center1,
                                           weight_center1, eccentricity, tick_, cur, prev, w, nullptr),
            "generateDoubleDiskCenter");
    } else {
      check(nbfmm_model_double_disk(k1, k2, center1, center2, radius1, radius2, weight, eccentricity, tick_, cur,
                                    prev, w, nullptr),
            "generateDoubleDisk");
    }
  } else if (!strcmp(model, "rectangle")) {
    if (argc <= 16) {
      cout << "Usage: " << argv[0] << " ... rectangle <rectangle width> <rectangle height> <maximum weight>" << endl
           << endl;
      abort();
    }
    const float model_width = atof(argv[14]);
    const float model_height = atof(argv[15]);
    const float max_weight = atof(argv[16]);
    printf("Model Rectangle: size = %.2f x %.2f, max weight = %.2f\n\n", model_width, model_height, max_weight);
    check(nbfmm_model_rectangle(num_star, center_position, model_width, model_height, max_weight, tick_, cur, prev,
                                w, nullptr),
          "generateRectangle");
  } else {
    cout << "Unknown model " << model << "." << endl;
    abort();
  }

  int progress = 0;
  for (int i = 0; i < 100; ++i) putchar('=');
  putchar('\r');
  fflush(stdout);

  nbfmm_movie* movie = nullptr;
  check(nbfmm_movie_open(stars, result_y4m, width, height, fps, size_scale, display_limits, &movie), "movie");
  check(nbfmm_movie_frame(movie, nullptr), "display");
  for (int j = 1; j < num_frame; ++j) {
    check(nbfmm_stars_update(stars, 1, nullptr), "update");
    check(nbfmm_movie_frame(movie, nullptr), "display");
    if (100 * j > progress * num_frame) {
      ++progress;
      putchar('>');
      fflush(stdout);
    }
  }
  putchar('\n');
  putchar('\n');
  check(nbfmm_movie_close(movie), "movie");
  check(nbfmm_stars_destroy(stars), "Stars");
  return 0;
}

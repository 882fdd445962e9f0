/*
 * A plain C99 host of the library's C ABI: no Python, no torch, only
 * include/dmgs.h and libdmgs_gb300.so — the way a non-Python caller binds the
 * rasteriser in place of the reference's `diff_gaussian_rasterization._C`.
 * It runs the host-side paths only (version, size queries, argument
 * validation, the derived FlexiCubes tables, the texture table layout), all
 * of which return before any CUDA call, so it needs no GPU.  The pointers
 * handed to the validating calls are never dereferenced.
 */
#include <stdio.h>
#include <string.h>

#include "dmgs.h"

static int failures = 0;
#define CHECK(c)                                                          \
  do {                                                                    \
    if (!(c)) {                                                           \
      fprintf(stderr, "%s:%d: check failed: %s (last error: %s)\n",      \
              __FILE__, __LINE__, #c, dmgs_last_error());                 \
      ++failures;                                                         \
    }                                                                     \
  } while (0)

static float fake[64]; /* stands for device arrays; 16-byte aligned use only */

static DmgsView view(void) {
  DmgsView v;
  memset(&v, 0, sizeof v);
  v.width = 64;
  v.height = 64;
  v.tanfovx = v.tanfovy = 0.5f;
  v.scale_modifier = 1.f;
  v.sh_degree = 3;
  v.bg = v.viewmatrix = v.projmatrix = v.campos = fake;
  return v;
}

static DmgsGaussians gaussians(void) {
  DmgsGaussians g;
  memset(&g, 0, sizeof g);
  g.P = 10;
  g.M = 16;
  g.means3D = g.opacities = g.shs = g.scales = g.rotations = fake;
  return g;
}

static int fwd(const DmgsView *v, const DmgsGaussians *g, size_t geom_bytes) {
  int64_t K = 0;
  return dmgs_raster_fwd_geometry(v, g, fake, geom_bytes, (int32_t *)fake, &K, NULL);
}

int main(void) {
  DmgsView v = view();
  DmgsGaussians g = gaussians();
  const size_t need = dmgs_geom_state_bytes(10, 64, 64);

  CHECK(dmgs_abi_version() == DMGS_ABI_VERSION);
  CHECK(need > 0 && need % 256 == 0);
  CHECK(dmgs_geom_state_bytes(2000, 256, 256) > dmgs_geom_state_bytes(1000, 256, 256));
  CHECK(dmgs_binning_state_bytes(1000000, 256, 256) > dmgs_binning_state_bytes(0, 256, 256));
  CHECK(dmgs_image_state_bytes(1237, 822) >= (size_t)1237 * 822 * 8);

  /* the reference's input-mode rules */
  g.shs = NULL;
  CHECK(fwd(&v, &g, need) == DMGS_ERR_ARG);
  CHECK(strstr(dmgs_last_error(), "exactly one of either SHs") != NULL);
  g = gaussians();
  g.cov3D_precomp = fake;
  CHECK(fwd(&v, &g, need) == DMGS_ERR_ARG);
  g = gaussians();
  g.M = 4; /* degree 3 needs 16 coefficients */
  CHECK(fwd(&v, &g, need) == DMGS_ERR_ARG);

  /* view validation and state sizes */
  g = gaussians();
  v.width = 0;
  CHECK(fwd(&v, &g, need) == DMGS_ERR_ARG);
  v = view();
  v.sh_degree = 4;
  CHECK(fwd(&v, &g, need) == DMGS_ERR_ARG);
  v = view();
  CHECK(fwd(&v, &g, need - 1) == DMGS_ERR_STATE);

  /* FlexiCubes: the derived Dual Marching Cubes tables (host only) */
  {
    uint16_t groups[1024];
    uint8_t nvd[256];
    int8_t chk[1280];
    int c, l, total = 0;
    CHECK(dmgs_fc_tables(groups, nvd, chk) == DMGS_OK);
    CHECK(nvd[0] == 0 && nvd[255] == 0 && nvd[1] == 1);
    for (c = 0; c < 256; ++c)
      for (l = 0; l < 4; ++l) total += groups[4 * c + l] != 0;
    {
      int vd = 0;
      for (c = 0; c < 256; ++c) vd += nvd[c];
      CHECK(total == vd); /* one non-empty edge group per dual vertex */
    }
  }
  {
    DmgsFcGrid fg;
    uint32_t counts[8];
    memset(&fg, 0, sizeof fg);
    fg.x = fg.s = fake;
    fg.rx = 0;
    fg.ry = fg.rz = 4;
    CHECK(dmgs_fc_count(&fg, fake, 1 << 20, counts, NULL) == DMGS_ERR_ARG);
  }

  /* hash-grid texture: table layout and validation */
  CHECK(dmgs_tex_table_entries(1.4473692f) > (1 << 19));
  CHECK(dmgs_tex_table_entries(0.5f) == -1);
  CHECK(dmgs_tex_bwd_scratch_bytes(10) == 10 * 128);
  CHECK(dmgs_sh_colors_fwd(10, 4, 25, fake, fake, fake, fake, NULL) == DMGS_ERR_ARG);

  if (failures == 0) printf("c consumer ok\n");
  return failures == 0 ? 0 : 1;
}

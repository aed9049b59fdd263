// apcomp_shim.cpp — C entry point over the reference's own partial
// compositor, apcomp::PartialCompositor<apcomp::VolumePartial<float>>
// (Ascent src/libs/apcomp/partial_compositor.cpp, the serial twin of
// vtkh/compositing/PartialCompositor.cpp).
//
// TEST INFRASTRUCTURE ONLY: this shim and the reference sources it is
// linked with are built into oracle/_ref/ by oracle/Makefile, and only
// tests load the result, to pin the compositing step of the oracle.
#include <apcomp/partial_compositor.hpp>
#include <vector>

struct ref_partial {
  int pixel_id;
  float depth;
  float rgb[3];
  float alpha;
};

extern "C" int ref_apcomp_composite(int n_images, const int *counts,
                                    const ref_partial *in, ref_partial *out)
{
  std::vector<std::vector<apcomp::VolumePartial<float>>> images(n_images);
  int off = 0;
  for (int i = 0; i < n_images; ++i) {
    images[i].resize(counts[i]);
    for (int k = 0; k < counts[i]; ++k) {
      const ref_partial &r = in[off + k];
      apcomp::VolumePartial<float> &p = images[i][k];
      p.m_pixel_id = r.pixel_id;
      p.m_depth = r.depth;
      p.m_pixel[0] = r.rgb[0];
      p.m_pixel[1] = r.rgb[1];
      p.m_pixel[2] = r.rgb[2];
      p.m_alpha = r.alpha;
    }
    off += counts[i];
  }
  std::vector<apcomp::VolumePartial<float>> res;
  apcomp::PartialCompositor<apcomp::VolumePartial<float>> compositor;
  compositor.composite(images, res);
  for (size_t k = 0; k < res.size(); ++k) {
    out[k].pixel_id = res[k].m_pixel_id;
    out[k].depth = res[k].m_depth;
    out[k].rgb[0] = res[k].m_pixel[0];
    out[k].rgb[1] = res[k].m_pixel[1];
    out[k].rgb[2] = res[k].m_pixel[2];
    out[k].alpha = res[k].m_alpha;
  }
  return (int)res.size();
}

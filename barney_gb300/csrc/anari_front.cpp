// anari_front.cpp -- the reference ANARI device's parameter translation for
// structuredRegular fields and transferFunction1D volumes
// (include/gbv_anari.h), over the bn* API.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/gbv_anari.h"
#include "gbv_internal.h"

using gbv::set_error;

extern "C" {

gbv_status gbv_anari_structured_regular_bounds(const int dims[3], const float origin[3], const float spacing[3],
                                               float lower[3], float upper[3]) {
  if (!dims || !lower || !upper) return set_error(GBV_ERROR_INVALID_ARGUMENT, "anari bounds: null pointer");
  for (int i = 0; i < 3; i++) {
    const float o = origin ? origin[i] : 0.f, s = spacing ? spacing[i] : 1.f;
    lower[i] = o;
    upper[i] = o + ((float)dims[i] - 1.f) * s;
  }
  return GBV_OK;
}

gbv_status gbv_anari_structured_regular(BNContext context, int slot, int element_type, const void *data,
                                        const int dims[3], const float origin[3], const float spacing[3],
                                        BNScalarField *field) {
  if (!context || !field) return set_error(GBV_ERROR_INVALID_ARGUMENT, "structuredRegular: null context or field");
  // a field without data is skipped with a warning (SpatialField.cpp:85-89)
  if (!data || !dims) return set_error(GBV_ERROR_INVALID_ARGUMENT,
                                       "missing required parameter 'data' on 'structuredRegular' field");
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "structuredRegular: empty data array");
  BNDataType type;
  switch (element_type) {
    case GBV_ANARI_FLOAT32: type = BN_FLOAT; break;
    case GBV_ANARI_UFIXED8:
    case GBV_ANARI_UINT8: type = BN_UFIXED8; break;
    default: return set_error(GBV_ERROR_UNSUPPORTED, "structuredRegular: scalar type not implemented");
  }
  if (!*field) *field = bnScalarFieldCreate(context, slot, "structured");
  if (!*field) return set_error(GBV_ERROR_INVALID_ARGUMENT, "structuredRegular: bnScalarFieldCreate failed");
  BNTextureData td = bnTextureData3DCreate(context, slot, type, dims[0], dims[1], dims[2], data);
  if (!td) return set_error(GBV_ERROR_INVALID_ARGUMENT, "structuredRegular: bnTextureData3DCreate failed");
  bnSetObject(*field, "textureData", td);
  bnRelease(td);
  bnSet3i(*field, "dims", dims[0], dims[1], dims[2]);
  bnSet3f(*field, "gridOrigin", origin ? origin[0] : 0.f, origin ? origin[1] : 0.f, origin ? origin[2] : 0.f);
  bnSet3f(*field, "gridSpacing", spacing ? spacing[0] : 1.f, spacing ? spacing[1] : 1.f,
          spacing ? spacing[2] : 1.f);
  bnCommit(*field);
  return GBV_OK;
}

float gbv_anari_density_scale(float unit_distance) { return unit_distance <= 0.f ? 1.f : 1.f / unit_distance; }

gbv_status gbv_anari_tf1d_rgba_map(const float *color, int color_channels, long long num_colors,
                                   const float *opacity, long long num_opacities, const float uniform_color[4],
                                   float opacity_param, float *rgba, long long *tf_size) {
  if (!tf_size) return set_error(GBV_ERROR_INVALID_ARGUMENT, "transferFunction1D: null size pointer");
  if (color && color_channels != 3 && color_channels != 4)
    return set_error(GBV_ERROR_UNSUPPORTED, "transferFunction1D: color arrays are vec3 or vec4 floats");
  if ((color && num_colors < 1) || (opacity && num_opacities < 1))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "transferFunction1D: empty color or opacity array");
  // Volume.cpp:95-99: uniform color (vec3 or vec4, default 1) and opacity
  float uc[4] = {1.f, 1.f, 1.f, 1.f};
  if (uniform_color) std::memcpy(uc, uniform_color, sizeof uc);
  const float uniformOpacity = opacity_param * uc[3];
  const long long numColors = color ? num_colors : 1;
  const long long numOpacities = opacity ? num_opacities : 1;
  const long long n = numColors > numOpacities ? numColors : numOpacities;
  *tf_size = n;
  if (!rgba) return GBV_OK;
  // Volume.cpp:136-170
  for (long long i = 0; i < n; ++i) {
    const float colorPos = n > 1 ? ((float)i / (float)(n - 1)) * (float)(numColors - 1) : 0.f;
    const float colorFrac = colorPos - floorf(colorPos);
    float c0[4] = {uc[0], uc[1], uc[2], uniformOpacity};
    float c1[4] = {uc[0], uc[1], uc[2], uniformOpacity};
    if (color) {
      const long long k0 = (long long)floorf(colorPos), k1 = (long long)ceilf(colorPos);
      if (color_channels == 3) {
        for (int a = 0; a < 3; a++) {
          c0[a] = color[3 * k0 + a];
          c1[a] = color[3 * k1 + a];
        }
      } else {
        for (int a = 0; a < 4; a++) {
          c0[a] = color[4 * k0 + a];
          c1[a] = color[4 * k1 + a];
        }
      }
    }
    float c[4];
    for (int a = 0; a < 4; a++) c[a] = (1.f - colorFrac) * c0[a] + colorFrac * c1[a];
    if (opacity) {
      const float alphaPos = n > 1 ? ((float)i / (float)(n - 1)) * (float)(numOpacities - 1) : 0.f;
      const float alphaFrac = alphaPos - floorf(alphaPos);
      const float a0 = opacity[(long long)floorf(alphaPos)], a1 = opacity[(long long)ceilf(alphaPos)];
      c[3] *= (1.f - alphaFrac) * a0 + alphaFrac * a1;
    }
    for (int a = 0; a < 4; a++) rgba[4 * i + a] = c[a];
  }
  return GBV_OK;
}

gbv_status gbv_anari_transfer_function_1d(BNVolume volume, const float *color, int color_channels,
                                          long long num_colors, const float *opacity, long long num_opacities,
                                          const float uniform_color[4], float opacity_param,
                                          const float value_range[2], float unit_distance, int user_id) {
  if (!volume) return set_error(GBV_ERROR_INVALID_ARGUMENT, "transferFunction1D: null volume");
  long long n = 0;
  gbv_status st = gbv_anari_tf1d_rgba_map(color, color_channels, num_colors, opacity, num_opacities, uniform_color,
                                          opacity_param, nullptr, &n);
  if (st != GBV_OK) return st;
  if (n > (1ll << 30)) return set_error(GBV_ERROR_INVALID_ARGUMENT, "transferFunction1D: map too large");
  std::vector<float> map((size_t)n * 4);
  st = gbv_anari_tf1d_rgba_map(color, color_channels, num_colors, opacity, num_opacities, uniform_color,
                               opacity_param, map.data(), &n);
  if (st != GBV_OK) return st;
  // valueRange default [0, 1] (Volume.cpp:94)
  bn_float2 range{value_range ? value_range[0] : 0.f, value_range ? value_range[1] : 1.f};
  bnSet1i(volume, "userID", user_id);
  bnVolumeSetXF(volume, range, reinterpret_cast<const bn_float4 *>(map.data()), (int)n,
                gbv_anari_density_scale(unit_distance));
  bnCommit(volume);
  return GBV_OK;
}

BNDataType gbv_anari_frame_color_format(int color_type) {
  switch (color_type) {
    case GBV_ANARI_UFIXED8_VEC4: return BN_UFIXED8_RGBA;
    case GBV_ANARI_UFIXED8_RGBA_SRGB: return BN_UFIXED8_RGBA_SRGB;
    case GBV_ANARI_FLOAT32: return BN_FLOAT;
    case GBV_ANARI_FLOAT32_VEC3: return BN_FLOAT32_VEC3;
    case GBV_ANARI_FLOAT32_VEC4: return BN_FLOAT4;
  }
  return BN_DATA_UNDEFINED;
}

uint32_t gbv_anari_frame_channels(int depth_type, int primitive_id_type, int object_id_type, int instance_id_type,
                                  int normal_type) {
  uint32_t c = BN_FB_COLOR;
  if (depth_type == GBV_ANARI_FLOAT32) c |= BN_FB_DEPTH;
  if (primitive_id_type == GBV_ANARI_UINT32) c |= BN_FB_PRIMID;
  if (object_id_type == GBV_ANARI_UINT32) c |= BN_FB_OBJID;
  if (instance_id_type == GBV_ANARI_UINT32) c |= BN_FB_INSTID;
  if (normal_type == GBV_ANARI_FLOAT32_VEC3) c |= BN_FB_NORMAL;
  return c;
}

gbv_status gbv_anari_frame_resize(BNFrameBuffer fb, int color_type, int depth_type, int primitive_id_type,
                                  int object_id_type, int instance_id_type, int normal_type, int width,
                                  int height) {
  if (!fb) return set_error(GBV_ERROR_INVALID_ARGUMENT, "anari frame: null frame buffer");
  if (width <= 0 || height <= 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "anari frame: empty size");
  const BNDataType fmt = gbv_anari_frame_color_format(color_type);
  if (fmt != BN_FLOAT4 && fmt != BN_UFIXED8_RGBA && fmt != BN_UFIXED8_RGBA_SRGB)
    return set_error(GBV_ERROR_UNSUPPORTED, "anari frame: color channel type other than UFIXED8_VEC4, "
                                            "UFIXED8_RGBA_SRGB or FLOAT32_VEC4");
  const uint32_t channels =
      gbv_anari_frame_channels(depth_type, primitive_id_type, object_id_type, instance_id_type, normal_type);
  if (channels & BN_FB_NORMAL) return set_error(GBV_ERROR_UNSUPPORTED, "anari frame: no normal channel on this path");
  bnFrameBufferResize(fb, fmt, width, height, channels);
  return GBV_OK;
}

}  // extern "C"

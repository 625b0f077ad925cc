/* gbv_anari.h -- the parameter translation of the reference's ANARI device
 * for the structured-volume path, as host functions over the bn* API.
 *
 * The reference's ANARI device (anari/, built on the ANARI SDK's helium
 * layer) turns a `structuredRegular` spatial field and a
 * `transferFunction1D` volume into barney objects on commit.  The SDK is not
 * needed for that translation: these functions take the committed ANARI
 * parameters as plain values (the arrays' data, element types and sizes) and
 * make the same bn* calls the reference's device makes, so an ANARI device
 * built on this library (or an app that holds ANARI-style parameters) gets
 * the reference's fields and transfer functions.  Each function cites the
 * reference code it replaces.  No call throws; a failure returns a status
 * and sets gbv_last_error() (errors of the bn* calls themselves go to
 * bnGetLastError(), as for any bn* call).
 */
#ifndef GBV_ANARI_H
#define GBV_ANARI_H
#include "barney_gb300.h"
#include "gbvol.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Element types of a structuredRegular field's `data` array that the
   reference's device accepts (ANARI_FLOAT32, ANARI_UFIXED8, ANARI_UINT8);
   any other type is rejected, as there (anari/SpatialField.cpp:105-116). */
enum { GBV_ANARI_FLOAT32 = 0, GBV_ANARI_UFIXED8 = 1, GBV_ANARI_UINT8 = 2 };

/* StructuredRegularField::finalize (anari/SpatialField.cpp:83-140): a
   "structured" bn scalar field with the data array as its texture data
   (FLOAT32 -> BN_FLOAT, UFIXED8/UINT8 -> BN_UFIXED8), "dims" = the array's
   size, "gridOrigin" = origin (null: 0) and "gridSpacing" = spacing (null:
   1), committed.  *field: an existing field to update, or null to create
   one (createBarneyScalarField, :143-153) whose handle is returned there. */
gbv_status gbv_anari_structured_regular(BNContext context, int slot, int element_type, const void *data,
                                        const int dims[3], const float origin[3], const float spacing[3],
                                        BNScalarField *field);

/* StructuredRegularField::bounds (anari/SpatialField.cpp:155-160):
   origin .. origin + (dims - 1) * spacing (null origin: 0, spacing: 1). */
gbv_status gbv_anari_structured_regular_bounds(const int dims[3], const float origin[3], const float spacing[3],
                                               float lower[3], float upper[3]);

/* The transferFunction1D's RGBA map (anari/Volume.cpp:129-170): tf_size =
   max(num_colors, num_opacities) entries (num 1 for an absent array); entry
   i interpolates the color array (color_channels 3 or 4; 0 = no array: the
   uniform color) and the opacity array (null: none) at their own positions
   i/(tf_size-1)*(num-1); the alpha is the color's alpha (vec4 colors) or the
   uniform opacity, times the interpolated opacity.  uniform_color (null:
   1,1,1,1) and opacity are the volume's "color" and "opacity" parameters;
   the uniform opacity is opacity * uniform_color[3] (:98-99).  With rgba ==
   null only *tf_size is returned. */
gbv_status gbv_anari_tf1d_rgba_map(const float *color, int color_channels, long long num_colors,
                                   const float *opacity, long long num_opacities, const float uniform_color[4],
                                   float opacity_param, float *rgba, long long *tf_size);

/* The density scale of a transferFunction1D: 1 / unitDistance, or 1 when
   unitDistance <= 0 (anari/Volume.cpp:113-119). */
float gbv_anari_density_scale(float unit_distance);

/* TransferFunction1D::finalize + setBarneyParameters (anari/Volume.cpp:
   107-127, 200-212): the RGBA map above, then on `volume` "userID" =
   user_id, bnVolumeSetXF(value_range, map, density scale), committed. */
gbv_status gbv_anari_transfer_function_1d(BNVolume volume, const float *color, int color_channels,
                                          long long num_colors, const float *opacity, long long num_opacities,
                                          const float uniform_color[4], float opacity_param,
                                          const float value_range[2], float unit_distance, int user_id);

/* Element types of an ANARI frame's channels ("channel.color",
   "channel.depth", "channel.primitiveId", "channel.objectId",
   "channel.instanceId", "channel.normal"); GBV_ANARI_UNKNOWN: the channel
   is not set. */
enum {
  GBV_ANARI_UNKNOWN = -1,
  GBV_ANARI_UFIXED8_VEC4 = 10,
  GBV_ANARI_UFIXED8_RGBA_SRGB = 11,
  GBV_ANARI_FLOAT32_VEC3 = 12,
  GBV_ANARI_FLOAT32_VEC4 = 13,
  GBV_ANARI_UINT32 = 14
};

/* toBarney (anari/Frame.cpp:20-35): the bn color format of a "channel.color"
   type -- UFIXED8_VEC4 -> BN_UFIXED8_RGBA, UFIXED8_RGBA_SRGB ->
   BN_UFIXED8_RGBA_SRGB, FLOAT32 -> BN_FLOAT, FLOAT32_VEC3 -> BN_FLOAT3,
   FLOAT32_VEC4 -> BN_FLOAT4, anything else BN_DATA_UNDEFINED. */
BNDataType gbv_anari_frame_color_format(int color_type);

/* Frame::finalize's requiredChannels (anari/Frame.cpp:108-120): BN_FB_COLOR,
   plus BN_FB_DEPTH for a FLOAT32 depth channel, BN_FB_PRIMID, BN_FB_OBJID,
   BN_FB_INSTID for UINT32 ID channels, BN_FB_NORMAL for a FLOAT32_VEC3
   normal channel. */
uint32_t gbv_anari_frame_channels(int depth_type, int primitive_id_type, int object_id_type, int instance_id_type,
                                  int normal_type);

/* Frame::finalize (anari/Frame.cpp:86-140) on the frame buffer: resize to
   width x height with the color format and channels above.  The frame's
   channels are then read as the reference's Frame::map reads them
   (anari/Frame.cpp:232-300): bnFrameBufferRead(fb, BN_FB_COLOR, ..., the
   color format), BN_FB_DEPTH as BN_FLOAT, the IDs as BN_INT32.  This path
   renders no normal channel: a FLOAT32_VEC3 normal channel is refused. */
gbv_status gbv_anari_frame_resize(BNFrameBuffer fb, int color_type, int depth_type, int primitive_id_type,
                                  int object_id_type, int instance_id_type, int normal_type, int width,
                                  int height);

#ifdef __cplusplus
}
#endif
#endif /* GBV_ANARI_H */

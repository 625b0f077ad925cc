/* barney_gb300.h -- barney-compatible C API for the structured-volume path.
 *
 * A drop-in for the subset of the reference's public API
 * (barney/include/barney.h, Barney 1.1.8) that renders a "structured"
 * scalar field with a transfer function on a single-GPU context: an app
 * linking libbarney_gb300.so in place of libbarney gets the same handles,
 * parameter names, data types and call sequence.  Names, enum values and
 * signatures below are those of barney.h; each function cites the line it
 * mirrors.
 *
 * Scope: one structured volume per model, identity instance transforms,
 * directional and env-map lights, perspective cameras, FLOAT4 / RGBA8 /
 * sRGB-RGBA8 color channels.  Calls outside that scope record an error
 * (bnGetLastError) and leave the object unchanged; no call throws.
 */
#ifndef BARNEY_GB300_H
#define BARNEY_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define BARNEY_API extern "C"
#define BN_IF_CPP(a) a
#else
#define BARNEY_API
#define BN_IF_CPP(a)
#endif

/* handle types (barney.h:58-77) */
#ifdef __cplusplus
typedef struct _BNContext *BNContext;
typedef struct _BNObject {} *BNObject;
typedef struct _BNData : public _BNObject {} *BNData;
typedef struct _BNTextureData : public _BNObject {} *BNTextureData;
typedef struct _BNScalarField : public _BNObject {} *BNScalarField;
typedef struct _BNGeom : public _BNObject {} *BNGeom;
typedef struct _BNVolume : public _BNObject {} *BNVolume;
typedef struct _BNGroup : public _BNObject {} *BNGroup;
typedef struct _BNModel : public _BNObject {} *BNModel;
typedef struct _BNRenderer : public _BNObject {} *BNRenderer;
typedef struct _BNFrameBuffer : public _BNObject {} *BNFrameBuffer;
typedef struct _BNTexture2D : public _BNObject {} *BNTexture2D;
typedef struct _BNTexture3D : public _BNObject {} *BNTexture3D;
typedef struct _BNLight : public _BNObject {} *BNLight;
typedef struct _BNCamera : public _BNObject {} *BNCamera;
typedef struct _BNMaterial : public _BNObject {} *BNMaterial;
typedef struct _BNSampler : public _BNObject {} *BNSampler;
#else
typedef struct _BNContext *BNContext;
typedef void *BNObject;
typedef void *BNData;
typedef void *BNTextureData;
typedef void *BNScalarField;
typedef void *BNGeom;
typedef void *BNVolume;
typedef void *BNGroup;
typedef void *BNModel;
typedef void *BNRenderer;
typedef void *BNFrameBuffer;
typedef void *BNTexture2D;
typedef void *BNTexture3D;
typedef void *BNLight;
typedef void *BNCamera;
typedef void *BNMaterial;
typedef void *BNSampler;
#endif
typedef BNTexture2D BNTexture;

/* barney.h:79-93 */
struct bn_float2 { float x, y; };
struct bn_float3 { float x, y, z; };
struct bn_float4 { float x, y, z, w; };
struct bn_int2 { int x, y; };
struct bn_int3 { int x, y, z; };
struct bn_int4 { int x, y, z, w; };
typedef struct bn_float2 bn_float2;
typedef struct bn_float3 bn_float3;
typedef struct bn_float4 bn_float4;
typedef struct BNTransform {
  struct { bn_float3 vx, vy, vz; } l;
  bn_float3 p;
} BNTransform;

/* barney.h:95-102 */
typedef enum {
  BN_FB_COLOR = (1 << 0),
  BN_FB_DEPTH = (1 << 1),
  BN_FB_PRIMID = (1 << 2),
  BN_FB_INSTID = (1 << 3),
  BN_FB_OBJID = (1 << 4),
  BN_FB_NORMAL = (1 << 5)
} BNFrameBufferChannel;

/* barney.h:104-179 (the values this path reads) */
typedef enum {
  BN_DATA_UNDEFINED = 0,
  BN_DATA,
  BN_OBJECT,
  BN_TEXTURE,
  BN_TEXTURE_3D,
  BN_UINT8 = 110,
  BN_UINT16 = 130,
  BN_INT32 = 140,
  BN_UINT32 = 150,
  BN_FLOAT32 = 180,
  BN_FLOAT32_VEC2,
  BN_FLOAT32_VEC3,
  BN_FLOAT32_VEC4,
  BN_FLOAT = BN_FLOAT32,
  BN_FLOAT4 = BN_FLOAT32_VEC4,
  BN_INT = BN_INT32,
  BN_UFIXED8 = 300,
  BN_UFIXED8_RGBA,
  BN_UFIXED8_RGBA_SRGB,
  BN_UFIXED16
} BNDataType;

/* barney.h:194-213 */
typedef enum { BN_TEXTURE_NEAREST, BN_TEXTURE_LINEAR } BNTextureFilterMode;
typedef enum { BN_TEXTURE_WRAP, BN_TEXTURE_CLAMP, BN_TEXTURE_BORDER, BN_TEXTURE_MIRROR } BNTextureAddressMode;
typedef enum { BN_COLOR_SPACE_LINEAR, BN_COLOR_SPACE_SRGB } BNTextureColorSpace;

/* context (barney.h:311-348) */
BARNEY_API BNContext bnContextCreate(const int *dataRanksOnThisContext BN_IF_CPP(= 0),
                                     int numDataRanksOnThisContext BN_IF_CPP(= 1),
                                     const int *gpuIDs BN_IF_CPP(= nullptr), int numGPUs BN_IF_CPP(= -1));
BARNEY_API void bnContextDestroy(BNContext context);
BARNEY_API void bnRelease(BNObject object);
BARNEY_API void bnAddReference(BNObject object);

/* object creation (barney.h:241-258, 421-533) */
BARNEY_API BNCamera bnCameraCreate(BNContext context, const char *type);
BARNEY_API BNFrameBuffer bnFrameBufferCreate(BNContext context, int deprecated BN_IF_CPP(= 0));
BARNEY_API BNModel bnModelCreate(BNContext ctx);
BARNEY_API BNRenderer bnRendererCreate(BNContext ctx, const char *type BN_IF_CPP(= "default"));
BARNEY_API BNData bnDataCreate(BNContext context, int whichSlot, BNDataType dataType, size_t numItems,
                               const void *items);
BARNEY_API BNTextureData bnTextureData3DCreate(BNContext context, int whichSlot, BNDataType texelFormat,
                                               int width, int height, int depth, const void *items);
/* barney.h:428: new contents for a data array (same element type) */
BARNEY_API void bnDataSet(BNData data, size_t numItems, const void *items);
/* barney.h:436, 476-488, 518: image textures and samplers for material
   parameters.  This path renders constant material parameters only: the
   objects are made (an ANARI device creates them for its samplers) and a
   material that is given one refuses it with a recorded message. */
BARNEY_API BNTextureData bnTextureData2DCreate(BNContext context, int whichSlot, BNDataType texelFormat,
                                               int width, int height, const void *items);
BARNEY_API BNTexture3D bnTexture3DCreate(BNContext context, int whichSlot, BNDataType texelFormat,
                                         uint32_t size_x, uint32_t size_y, uint32_t size_z, const void *texels,
                                         BNTextureFilterMode filterMode BN_IF_CPP(= BN_TEXTURE_LINEAR),
                                         BNTextureAddressMode addressMode BN_IF_CPP(= BN_TEXTURE_CLAMP));
BARNEY_API BNSampler bnSamplerCreate(BNContext context, int whichSlot, const char *type);
BARNEY_API BNTexture2D bnTexture2DCreate(BNContext context, int whichSlot, BNDataType texelFormat,
                                         uint32_t size_x, uint32_t size_y, const void *texels,
                                         BNTextureFilterMode filterMode BN_IF_CPP(= BN_TEXTURE_LINEAR),
                                         BNTextureAddressMode addressMode_x BN_IF_CPP(= BN_TEXTURE_WRAP),
                                         BNTextureAddressMode addressMode_y BN_IF_CPP(= BN_TEXTURE_WRAP),
                                         BNTextureColorSpace colorSpace BN_IF_CPP(= BN_COLOR_SPACE_LINEAR));
BARNEY_API BNLight bnLightCreate(BNContext context, int whichSlot, const char *type);
/* "iso_surface" (IsoSurface: "scalarField", "isoValue", "material"); other
   geometry types are outside this path and return 0 (barney.h:498-500,
   barney/geometry/Geometry.cpp:26-43) */
BARNEY_API BNGeom bnGeometryCreate(BNContext context, int whichSlot, const char *type);
/* "matte" / "AnariMatte" (constant "color" and "opacity"); other material
   types return 0 (barney.h:513-516, barney/material/Material.cpp:83-98) */
BARNEY_API BNMaterial bnMaterialCreate(BNContext context, int whichSlot, const char *type);
BARNEY_API BNGroup bnGroupCreate(BNContext context, int whichSlot, BNGeom *geoms, int numGeoms,
                                 BNVolume *volumes, int numVolumes);
BARNEY_API void bnGroupBuild(BNGroup group);
BARNEY_API BNScalarField bnScalarFieldCreate(BNContext context, int whichSlot, const char *type);
BARNEY_API BNVolume bnVolumeCreate(BNContext context, int whichSlot, BNScalarField sf);
BARNEY_API void bnVolumeSetXF(BNVolume volume, bn_float2 domain, const bn_float4 *colorMap,
                              int numColorMapValues, float densityAt1);

/* parameters (barney.h:266-308) */
BARNEY_API void bnCommit(BNObject target);
BARNEY_API void bnSetString(BNObject target, const char *paramName, const char *value);
BARNEY_API void bnSetData(BNObject target, const char *paramName, BNData value);
BARNEY_API void bnSetObject(BNObject target, const char *paramName, const BNObject value);
BARNEY_API void bnSetLight(BNObject target, const char *paramName, BNLight value);
BARNEY_API void bnSet1i(BNObject target, const char *paramName, int value);
BARNEY_API void bnSet2i(BNObject target, const char *paramName, int x, int y);
BARNEY_API void bnSet3i(BNObject target, const char *paramName, int x, int y, int z);
BARNEY_API void bnSet4i(BNObject target, const char *paramName, int x, int y, int z, int w);
BARNEY_API void bnSet1f(BNObject target, const char *paramName, float value);
BARNEY_API void bnSet2f(BNObject target, const char *paramName, float x, float y);
BARNEY_API void bnSet3f(BNObject target, const char *paramName, float x, float y, float z);
BARNEY_API void bnSet4f(BNObject target, const char *paramName, float x, float y, float z, float w);
BARNEY_API void bnSet4x3fv(BNObject target, const char *paramName, const BNTransform *affineMatrix);
BARNEY_API void bnSet4x4fv(BNObject target, const char *paramName, const bn_float4 *xfm);

/* model and render (barney.h:351-390) */
BARNEY_API void bnSetInstances(BNModel model, int whichSlot, BNGroup *groupsToInstantiate,
                               BNTransform *instanceTransforms, int numInstances);
/* barney.h:397: new transforms for the instances bnSetInstances set */
BARNEY_API void bnUpdateInstanceTransforms(BNModel model, int whichSlot, BNTransform *instanceTransforms,
                                           int numInstances);
/* barney.h:405: per-instance attribute arrays ("instID", "attribute0".."4",
   "color"); kept with the model -- the reference's device code reads none
   of them on this path (its instance-ID map stays unset) */
BARNEY_API void bnSetInstanceAttributes(BNModel model, int whichSlot, const char *attributeName, BNData data);
BARNEY_API void bnBuild(BNModel model, int whichDataSlot);
BARNEY_API void bnAccumReset(BNFrameBuffer fb);
BARNEY_API void bnFrameBufferResize(BNFrameBuffer fb, BNDataType colorFormat, int sizeX, int sizeY,
                                    uint32_t requiredChannels BN_IF_CPP(= BN_FB_COLOR));
BARNEY_API void bnFrameBufferRead(BNFrameBuffer fb, BNFrameBufferChannel channelToRead,
                                  void *pointerToReadDataInto, BNDataType requiredFormat);
BARNEY_API void bnFrameBufferGetSize(BNFrameBuffer fb, int *sizeX, int *sizeY);
BARNEY_API void bnRender(BNRenderer renderer, BNModel model, BNCamera camera, BNFrameBuffer fb);

/* Additions of this library (no counterpart in barney.h). */
/* Message of the last failed bn* call on this thread ("" if none since the
   thread's last successful bnContextCreate, which starts it afresh). */
BARNEY_API const char *bnGetLastError(void);
/* Statistics of the last bnRender on this frame buffer: density samples,
   macrocells entered, rays traced, loop-cap events. */
BARNEY_API void bnFrameBufferGetStats(BNFrameBuffer fb, unsigned long long stats[4]);

#ifdef __cplusplus
/* barney.h:537-551: the C++ overloads over the typed setters */
inline void bnSet(BNObject o, const char *n, bn_float2 v) { bnSet2f(o, n, v.x, v.y); }
inline void bnSet(BNObject o, const char *n, bn_float3 v) { bnSet3f(o, n, v.x, v.y, v.z); }
inline void bnSet(BNObject o, const char *n, bn_float4 v) { bnSet4f(o, n, v.x, v.y, v.z, v.w); }
inline void bnSet(BNObject o, const char *n, bn_int2 v) { bnSet2i(o, n, v.x, v.y); }
inline void bnSet(BNObject o, const char *n, bn_int3 v) { bnSet3i(o, n, v.x, v.y, v.z); }
inline void bnSet(BNObject o, const char *n, bn_int4 v) { bnSet4i(o, n, v.x, v.y, v.z, v.w); }
#endif

#endif /* BARNEY_GB300_H */

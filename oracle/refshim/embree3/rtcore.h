// Stand-in for Embree 3's type names, declarations only: the reference's LBVH
// sources name these types but call no Embree function (test infrastructure).
#pragma once
typedef struct RTCDeviceTy *RTCDevice;
typedef struct RTCSceneTy *RTCScene;
typedef struct RTCGeometryTy *RTCGeometry;
enum RTCError { RTC_ERROR_NONE = 0 };
typedef void (*RTCErrorFunction)(void *userPtr, enum RTCError code, const char *str);
RTCDevice rtcNewDevice(const char *config);
enum RTCError rtcGetDeviceError(RTCDevice device);
void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction error, void *userPtr);

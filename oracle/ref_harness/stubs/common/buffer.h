// Stand-in for the reference's host/device buffer classes (declarations only).
#pragma once
template <typename T>
struct HostDeviceBuffer {};
template <typename T>
struct DeviceBuffer {};

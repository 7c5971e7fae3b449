/* PshPack1.h -- Windows SDK packing helper: push 1-byte structure packing. */
#pragma pack(push, 1)

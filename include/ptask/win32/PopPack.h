/* PopPack.h -- Windows SDK packing helper: restore the previous structure packing. */
#pragma pack(pop)

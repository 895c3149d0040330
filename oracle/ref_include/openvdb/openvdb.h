// openvdb/openvdb.h -- empty stand-in.  The reference's Heterogeneous
// medium includes OpenVDB for its OpenVDBVolume, which the pinned grid
// path (GridVolume) never touches.
#pragma once

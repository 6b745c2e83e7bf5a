// Stand-in for the reference's util::Image3D (flyingEdges/util/Image3D.h) in
// the shim test: the constructor and the accessors the shim reads.
#pragma once
#include <array>
#include <vector>

#include "FlyingEdges_Config.h"

namespace util {

class Image3D
{
public:
    Image3D(std::vector<scalar_t> data, std::array<scalar_t, 3> spacing, std::array<scalar_t, 3> zeroPos,
            std::array<size_t, 3> dims)
      : data_(std::move(data)), spacing_(spacing), zeroPos_(zeroPos), dims_(dims)
    {}
    const scalar_t* pointer() const { return data_.data(); }
    std::array<scalar_t, 3> getZeroPos() const { return zeroPos_; }
    std::array<scalar_t, 3> getSpacing() const { return spacing_; }
    size_t xdimension() const { return dims_[0]; }
    size_t ydimension() const { return dims_[1]; }
    size_t zdimension() const { return dims_[2]; }

private:
    std::vector<scalar_t> data_;
    std::array<scalar_t, 3> spacing_, zeroPos_;
    std::array<size_t, 3> dims_;
};

}  // namespace util

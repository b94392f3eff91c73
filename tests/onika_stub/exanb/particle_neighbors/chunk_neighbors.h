#pragma once
namespace exanb {
struct GridChunkNeighbors {};
}

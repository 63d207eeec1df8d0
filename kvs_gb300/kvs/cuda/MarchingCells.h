/*****************************************************************************/
/**
 *  @file   MarchingCells.h
 *  @brief  kvs::cuda::MarchingTetrahedra, MarchingHexahedra, MarchingPyramid
 *          and MarchingPrism -- GB300 drop-ins for the reference's
 *          unstructured marching mappers.
 *
 *  Same constructor, setIsolevel and exec(ObjectBase*) as the reference
 *  mappers (Source/Core/Visualization/Mapper/MarchingTetrahedra.h:23-60 and
 *  the three alike); each is a kvs::MapperBase and a kvs::PolygonObject with
 *  the reference's checks, messages, min/max cache, transfer-function range,
 *  bounding box and single polygon colour, and the same coordinate and normal
 *  bits.  Classification, interpolation, normals and the compaction in cell
 *  order run on the GPU (kvsmc_marching_cells_host).  As in the reference,
 *  isSuccess() is never set true, and duplication == false (forced by
 *  VertexNormal) extracts nothing.  When the GPU call fails, exec reports
 *  kvsMessageError and returns nullptr (no CPU fallback).
 */
/*****************************************************************************/
#pragma once
#include <kvs/MapperBase>
#include <kvs/Module>
#include <kvs/PolygonObject>
#include <kvs/UnstructuredVolumeObject>

namespace kvs
{

namespace cuda
{

/// UnstructuredVolumeObject::updateMinMaxCoords on the GPU (kvsmc_cells_bounds),
/// written into the volume's bounding box; false (and a message) on failure.
bool DeviceBounds( const kvs::UnstructuredVolumeObject* volume, int cell, int device );

/// The body the four mappers share; not a module itself.
class MarchingCellsBase : public kvs::MapperBase, public kvs::PolygonObject
{
public:
    typedef kvs::MapperBase BaseClass;
    typedef kvs::PolygonObject SuperClass;

protected:
    double m_isolevel = 0;     ///< isosurface level
    bool m_duplication = true; ///< duplication flag (sticky false after VertexNormal)
    int m_device = -1;         ///< CUDA device (-1: the current one)

    struct Traits
    {
        int cell;                                     ///< kvsmc_cell_type
        kvs::UnstructuredVolumeObject::CellType type; ///< the volume's cell type
        const char* type_message;                     ///< "Input volume is not ...-cell data."
        const char* dtype_message;                    ///< the unsupported-type message
        bool types_need_duplication;                  ///< tetrahedra set the types only with duplication
    };

    MarchingCellsBase() = default;
    MarchingCellsBase( const kvs::TransferFunction& transfer_function, double isolevel, bool duplication );

    SuperClass* run( const kvs::ObjectBase* object, const Traits& traits );

public:
    virtual ~MarchingCellsBase() = default;

    void setIsolevel( const double isolevel ) { m_isolevel = isolevel; }
    void setDevice( const int device ) { m_device = device; }
    /// the constructor's duplication flag, for the pipeline-module form
    void setDuplication( const bool duplication ) { m_duplication = duplication; }

private:
    bool mapping( const kvs::UnstructuredVolumeObject* volume, const Traits& traits );
};

#define KVSMC_CELL_MAPPER( NAME )                                                       \
    class NAME : public MarchingCellsBase                                               \
    {                                                                                   \
        kvsModule( kvs::cuda::NAME, Mapper );                                           \
        kvsModuleBaseClass( kvs::MapperBase );                                          \
        kvsModuleSuperClass( kvs::PolygonObject );                                      \
                                                                                        \
    public:                                                                             \
        NAME() = default;                                                               \
        virtual ~NAME() = default;                                                      \
        NAME( const kvs::UnstructuredVolumeObject* volume, const double isolevel,       \
              const SuperClass::NormalType normal_type, const bool duplication,         \
              const kvs::TransferFunction& transfer_function );                         \
        SuperClass* exec( const kvs::ObjectBase* object );                              \
    }

KVSMC_CELL_MAPPER( MarchingTetrahedra );
KVSMC_CELL_MAPPER( MarchingHexahedra );
KVSMC_CELL_MAPPER( MarchingPyramid );
KVSMC_CELL_MAPPER( MarchingPrism );

#undef KVSMC_CELL_MAPPER

} // end of namespace cuda

} // end of namespace kvs

/*****************************************************************************/
/**
 *  @file   MarchingCubes.h
 *  @brief  kvs::cuda::MarchingCubes -- GB300 drop-in for kvs::MarchingCubes.
 *
 *  Same constructor, setIsolevel and exec(ObjectBase*) as the reference mapper
 *  (Source/Core/Visualization/Mapper/MarchingCubes.h:23-62); it is a
 *  kvs::MapperBase and a kvs::PolygonObject, so it plugs into
 *  kvs::PipelineModule / kvs::VisualizationPipeline and returns the same
 *  PolygonObject arrays, bit for bit.  The per-cell work runs on the GPU
 *  through libkvsmc (include/kvsmc.h); there is no CPU fallback: when the GPU
 *  call fails, exec reports kvsMessageError, sets isSuccess() false and
 *  returns nullptr.
 */
/*****************************************************************************/
#pragma once
#include <kvs/MapperBase>
#include <kvs/Module>
#include <kvs/PolygonObject>
#include <kvs/StructuredVolumeObject>

namespace kvs
{

namespace cuda
{

class MarchingCubes : public kvs::MapperBase, public kvs::PolygonObject
{
    kvsModule( kvs::cuda::MarchingCubes, Mapper );
    kvsModuleBaseClass( kvs::MapperBase );
    kvsModuleSuperClass( kvs::PolygonObject );

private:
    double m_isolevel = 0;     ///< isosurface level
    bool m_duplication = true; ///< duplication flag (sticky false after VertexNormal)
    int m_device = -1;         ///< CUDA device (-1: the current one)

public:
    MarchingCubes() = default;
    virtual ~MarchingCubes() = default;

    MarchingCubes(
        const kvs::StructuredVolumeObject* volume,
        const double isolevel,
        const SuperClass::NormalType normal_type,
        const bool duplication,
        const kvs::TransferFunction& transfer_function );

    void setIsolevel( const double isolevel ) { m_isolevel = isolevel; }
    void setDevice( const int device ) { m_device = device; }
    /// the constructor's duplication flag, for the pipeline-module form
    void setDuplication( const bool duplication ) { m_duplication = duplication; }

    SuperClass* exec( const kvs::ObjectBase* object );

private:
    bool mapping( const kvs::StructuredVolumeObject* volume );
};

} // end of namespace cuda

} // end of namespace kvs

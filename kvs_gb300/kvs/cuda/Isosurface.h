/*****************************************************************************/
/**
 *  @file   Isosurface.h
 *  @brief  kvs::cuda::Isosurface -- kvs::Isosurface with its structured and
 *          unstructured branches on the GPU.
 *
 *  Same constructors, setIsolevel and exec(ObjectBase*) as the reference
 *  mapper (Source/Core/Visualization/Mapper/Isosurface.h:23-57).  A
 *  structured volume goes to kvs::cuda::MarchingCubes (libkvsmc) where the
 *  reference builds a kvs::MarchingCubes (Isosurface.cpp:176-191); the
 *  arrays are the same bit for bit.  Unstructured volumes go, by cell type,
 *  to kvs::cuda::MarchingTetrahedra / Hexahedra / Pyramid / Prism where the
 *  reference builds its own mappers (Isosurface.cpp:193-258).  When the GPU
 *  mapper fails, exec reports kvsMessageError and returns nullptr (no CPU
 *  fallback).
 */
/*****************************************************************************/
#pragma once
#include <kvs/MapperBase>
#include <kvs/Module>
#include <kvs/PolygonObject>
#include <kvs/VolumeObjectBase>

namespace kvs
{

namespace cuda
{

class Isosurface : public kvs::MapperBase, public kvs::PolygonObject
{
    kvsModule( kvs::cuda::Isosurface, Mapper );
    kvsModuleBaseClass( kvs::MapperBase );
    kvsModuleSuperClass( kvs::PolygonObject );

private:
    double m_isolevel = 0.0;   ///< isosurface level
    bool m_duplication = true; ///< duplication flag
    int m_device = -1;         ///< CUDA device (-1: the current one)

public:
    Isosurface() = default;
    Isosurface(
        const kvs::VolumeObjectBase* volume,
        const SuperClass::NormalType normal_type = SuperClass::PolygonNormal );
    Isosurface(
        const kvs::VolumeObjectBase* volume,
        const double isolevel,
        const SuperClass::NormalType normal_type = SuperClass::PolygonNormal );
    Isosurface(
        const kvs::VolumeObjectBase* volume,
        const double isolevel,
        const SuperClass::NormalType normal_type,
        const bool duplication,
        const kvs::TransferFunction& transfer_function );
    virtual ~Isosurface() = default;

    void setIsolevel( const double isolevel ) { m_isolevel = isolevel; }
    void setDevice( const int device ) { m_device = device; }

    SuperClass* exec( const kvs::ObjectBase* object );

private:
    bool mapping( const kvs::VolumeObjectBase* volume );
    void shallowCopy( const kvs::PolygonObject* polygon );
};

} // end of namespace cuda

} // end of namespace kvs

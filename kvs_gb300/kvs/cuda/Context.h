/*****************************************************************************/
/**
 *  @file   Context.h
 *  @brief  The libkvsmc context the kvs::cuda mappers share (one per host
 *          thread and device, kept for the thread's life), and the
 *          kvs value type -> kvsmc_dtype map.
 */
/*****************************************************************************/
#pragma once
#include <kvs/AnyValueArray>

#include "kvsmc.h"

namespace kvs
{
namespace cuda
{

/// The calling thread's context on `device` (-1: the current device); null
/// and *status set when it cannot be created (no GPU, no driver).
kvsmc_context* DeviceContext( int device, kvsmc_status* status );

/// kvsmc_dtype of a value array (the reference's type switch,
/// MarchingCubes.cpp:113-124), or -1 for a type the mapper does not take.
int DType( const kvs::AnyValueArray& values );

} // end of namespace cuda
} // end of namespace kvs

{-# LANGUAGE ForeignFunctionInterface #-}
{-# LANGUAGE ScopedTypeVariables      #-}
{-# LANGUAGE TypeApplications         #-}
-- |
-- Module      : Data.Array.Accelerate.Math.FFT.LLVM.PTX.SpecConv
--
-- GPU foreign functions for the spectral convolution
--
--   y_b = fft3D Inverse (fft3D Forward x_b * H),   b = 0 .. batch-1,
--
-- and its vector-Jacobian product, served by libgbfft's fused kernels
-- (gbfft_specconv_fwd / gbfft_specconv_bwd, include/gbfft.h).  The reference
-- has no such operation: it composes it from fft3D (FFT.hs:150-173) and a
-- zipWith, and has no derivative.  The VJP takes g_y = dL/dy and returns
-- (g_x, g_H) = (dL/dx, dL/dH) in the conjugate-Wirtinger convention, g_H
-- summed over the batch; the forward spectrum of x is recomputed on the GPU,
-- not stored.  Complex Float only (the library's kernels for this operation).
--
-- The module follows the foreign-function shape of PTX.hs (allocateRemote,
-- ptxStream, withArray, new/put); it is written against accelerate-llvm-ptx
-- 1.3 and has not been compiled here (no GHC in this environment).
--
module Data.Array.Accelerate.Math.FFT.LLVM.PTX.SpecConv (

  specConv,
  specConvVJP,

) where

import Data.Array.Accelerate.Math.FFT.LLVM.PTX.Base

import Data.Array.Accelerate.Lifetime
import Data.Array.Accelerate.Representation.Array
import Data.Array.Accelerate.Representation.Shape
import Data.Array.Accelerate.Sugar.Elt
import Data.Array.Accelerate.Data.Complex
import Data.Array.Accelerate.Math.FFT.Type
import Data.Primitive.Vec

import Data.Array.Accelerate.LLVM.PTX.Foreign

import Foreign.CUDA.Ptr                                             ( DevicePtr, useDevicePtr )
import qualified Foreign.CUDA.Driver.Stream                         as CUDA

import Control.Exception
import Control.Monad.Reader
import Data.IORef
import Data.Int
import qualified Data.Map.Strict                                    as Map
import Foreign.C.Types
import Foreign.Marshal.Alloc                                        ( alloca )
import Foreign.Ptr
import Foreign.Storable                                             ( peek )
import System.IO.Unsafe                                             ( unsafePerformIO )


-- Plan creation allocates device tables and synchronises: a safe call.
foreign import ccall safe "gbfft_specconv_plan_create"
  c_plan_create :: Ptr (Ptr ()) -> Int64 -> Int64 -> Int64 -> Int64 -> CInt -> IO CInt

-- The passes only enqueue work on the stream: unsafe calls.
foreign import ccall unsafe "gbfft_specconv_fwd"
  c_fwd :: Ptr () -> Ptr () -> Ptr () -> Ptr () -> Ptr () -> IO CInt

foreign import ccall unsafe "gbfft_specconv_bwd"
  c_bwd :: Ptr () -> Ptr () -> Ptr () -> Ptr () -> Ptr () -> Ptr () -> Ptr () -> IO CInt

newtype SpecConvException = SpecConvException Int
  deriving Show

instance Exception SpecConvException

check :: CInt -> IO ()
check r = when (r /= 0) $ throwIO (SpecConvException (fromIntegral r))

-- Plans per (batch, d, h, w), created on first use and kept for the life of
-- the process (the library's own plan cache does the same for fft plans).
{-# NOINLINE plans #-}
plans :: IORef (Map.Map (Int64, Int64, Int64, Int64) (Ptr ()))
plans = unsafePerformIO (newIORef Map.empty)

planFor :: (Int64, Int64, Int64, Int64) -> IO (Ptr ())
planFor key@(b, d, h, w) = do
  m <- readIORef plans
  case Map.lookup key m of
    Just p  -> return p
    Nothing -> alloca $ \pp -> do
      check =<< c_plan_create pp b d h w 0   -- GBFFT_C32
      p <- peek pp
      atomicModifyIORef' plans (\m' -> (Map.insert key p m', ()))
      return p

type Field  = Array DIM4 (Vec2 Float)   -- batch x d x h x w
type Filter = Array DIM3 (Vec2 Float)   -- d x h x w

dims4 :: DIM4 -> (Int64, Int64, Int64, Int64)
dims4 (((((), w), h), d), b) = (fromIntegral b, fromIntegral d, fromIntegral h, fromIntegral w)

fieldR :: ArrayR Field
fieldR = ArrayR dim4 (eltR @(Complex Float))

filterR :: ArrayR Filter
filterR = ArrayR dim3 (eltR @(Complex Float))

-- | y = specConv (x, H)
specConv :: ForeignAcc ((((), Field), Filter) -> Field)
specConv = ForeignAcc "gbfft.specconv.fwd" go
  where
    go (((), x), hf) = do
      let sh = shape x
      y      <- allocateRemote fieldR sh
      stream <- asks ptxStream
      future <- new
      liftPar $
        withArray NumericRfloat32 x  stream $ \dx ->
        withArray NumericRfloat32 hf stream $ \dh ->
        withArray NumericRfloat32 y  stream $ \dy ->
        liftIO $ withLifetime stream $ \s -> do
          p <- planFor (dims4 sh)
          check =<< c_fwd p (ptr dx) (ptr dh) (ptr dy) (castPtr (CUDA.useStream s))
      put future y
      return future

-- | (g_x, g_H) = specConvVJP (x, H, g_y)
specConvVJP :: ForeignAcc (((((), Field), Filter), Field) -> (((), Field), Filter))
specConvVJP = ForeignAcc "gbfft.specconv.vjp" go
  where
    go ((((), x), hf), gy) = do
      let sh = shape x
      gx     <- allocateRemote fieldR sh
      gh     <- allocateRemote filterR (shape hf)
      stream <- asks ptxStream
      future <- new
      liftPar $
        withArray NumericRfloat32 x  stream $ \dx  ->
        withArray NumericRfloat32 hf stream $ \dh  ->
        withArray NumericRfloat32 gy stream $ \dgy ->
        withArray NumericRfloat32 gx stream $ \dgx ->
        withArray NumericRfloat32 gh stream $ \dgh ->
        liftIO $ withLifetime stream $ \s -> do
          p <- planFor (dims4 sh)
          check =<< c_bwd p (ptr dx) (ptr dh) (ptr dgy) (ptr dgx) (ptr dgh) (castPtr (CUDA.useStream s))
      put future (((), gx), gh)
      return future

ptr :: DevicePtr a -> Ptr ()
ptr = castPtr . useDevicePtr

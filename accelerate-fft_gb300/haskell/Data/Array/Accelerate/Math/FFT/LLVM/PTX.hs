{-# LANGUAGE FlexibleContexts    #-}
{-# LANGUAGE ForeignFunctionInterface #-}
{-# LANGUAGE GADTs               #-}
{-# LANGUAGE ScopedTypeVariables #-}
{-# LANGUAGE TypeApplications    #-}
{-# LANGUAGE TypeOperators       #-}
-- |
-- Module      : Data.Array.Accelerate.Math.FFT.LLVM.PTX
--
-- Drop-in replacement for accelerate-fft's GPU foreign path
-- (src/Data/Array/Accelerate/Math/FFT/LLVM/PTX.hs in accelerate-fft 1.3):
-- the same four exports with the same types, served by libgbfft (the
-- GB300 kernels, C ABI in include/gbfft.h) instead of cuFFT.
--
-- What changes relative to the cuFFT module:
--
--   * withPlan ... cuFFT (PTX.hs:98-124) becomes two foreign calls.  The
--     plan lookup, gbfft_plan_get, is imported `safe`: on a cache miss it
--     builds the plan (and may time candidates with GBFFT_AUTOTUNE=1),
--     which synchronises the device and can take seconds, so it must not
--     block the GHC capability.  The cache is the library's own, keyed on
--     the CUDA context and the full shape rather than a hash.  The launch,
--     gbfft_exec, only enqueues kernels on the Accelerate stream and is
--     imported `unsafe`.  No setStream: the stream is an argument, so
--     concurrent uses of one plan are safe.
--   * Inverse is normalised inside the kernels, and ranks 4 and 5 of `fft`
--     run here too.  FFT.hs therefore divides only on the paths that do not
--     normalise, and its PTX rank guard goes from 3 to 5 (FFT.hs.patch,
--     next to this module, makes both changes).
--   * PTX/Plans.hs and the cufft dependency are no longer needed;
--     PTX/Base.hs (withArray, waypoint) is reused unchanged.
--
module Data.Array.Accelerate.Math.FFT.LLVM.PTX (

  fft,
  fft1D,
  fft2D,
  fft3D,

) where

import Data.Array.Accelerate.Math.FFT.Mode
import Data.Array.Accelerate.Math.FFT.Type
import Data.Array.Accelerate.Math.FFT.LLVM.PTX.Base

import Data.Array.Accelerate.Analysis.Match
import Data.Array.Accelerate.Error
import Data.Array.Accelerate.Lifetime
import Data.Array.Accelerate.Representation.Array
import Data.Array.Accelerate.Representation.Shape
import Data.Array.Accelerate.Sugar.Elt
import Data.Array.Accelerate.Data.Complex
import Data.Primitive.Vec

import Data.Array.Accelerate.LLVM.PTX.Foreign

import Foreign.CUDA.Ptr                                             ( DevicePtr, useDevicePtr )
import qualified Foreign.CUDA.Driver.Stream                         as CUDA

import Control.Exception
import Control.Monad.Reader
import Data.Int
import Foreign.C.Types
import Foreign.Marshal.Alloc                                        ( alloca )
import Foreign.Marshal.Array                                        ( withArrayLen )
import Foreign.Storable                                             ( peek )
import Foreign.Ptr


-- | Cached plan lookup (gbfft.h, gbfft_plan_get): may build and tune a
-- plan on a miss, so it is a safe call.
foreign import ccall safe "gbfft_plan_get"
  c_gbfft_plan_get :: Ptr (Ptr ()) -> CInt -> Ptr Int64 -> CInt -> CInt -> CInt -> IO CInt

-- | Enqueue a plan's kernels on a stream (gbfft.h, gbfft_exec): no host
-- synchronisation, so an unsafe call.
foreign import ccall unsafe "gbfft_exec"
  c_gbfft_exec :: Ptr () -> CInt -> Ptr () -> Ptr () -> Ptr () -> IO CInt

foreign import ccall unsafe "gbfft_error_string"
  c_gbfft_error_string :: CInt -> IO (Ptr CChar)

data GbfftException = GbfftException !Int
  deriving Show

instance Exception GbfftException


fft :: forall sh e. HasCallStack
    => Mode
    -> ShapeR sh
    -> NumericR e
    -> ForeignAcc (Array sh (Vec2 e) -> Array sh (Vec2 e))
fft mode shR eR
  | Just Refl <- matchShapeR shR dim1 = fft1D mode eR
  | Just Refl <- matchShapeR shR dim2 = ForeignAcc "gbfft.fft2.many" $ fft' kindMany mode shR eR
  | Just Refl <- matchShapeR shR dim3 = ForeignAcc "gbfft.fft3.many" $ fft' kindMany mode shR eR
  -- ranks 4 and 5 (the reference falls back to its pure transform, FFT.hs:78)
  | rank shR <= 5 = ForeignAcc ("gbfft.fft" ++ show (rank shR) ++ ".many") $ fft' kindMany mode shR eR
  | otherwise = internalError "only for 1D..5D inner-dimension transforms"

fft1D :: Mode -> NumericR e -> ForeignAcc (Array DIM1 (Vec2 e) -> Array DIM1 (Vec2 e))
fft1D mode eR = ForeignAcc "gbfft.fft1d" $ fft' kindFull mode dim1 eR

fft2D :: Mode -> NumericR e -> ForeignAcc (Array DIM2 (Vec2 e) -> Array DIM2 (Vec2 e))
fft2D mode eR = ForeignAcc "gbfft.fft2d" $ fft' kindFull mode dim2 eR

fft3D :: Mode -> NumericR e -> ForeignAcc (Array DIM3 (Vec2 e) -> Array DIM3 (Vec2 e))
fft3D mode eR = ForeignAcc "gbfft.fft3d" $ fft' kindFull mode dim3 eR


-- Internals
-- ---------

kindMany, kindFull :: CInt
kindMany = 0    -- GBFFT_KIND_MANY
kindFull = 1    -- GBFFT_KIND_FULL

-- GBFFT_FORWARD / GBFFT_REVERSE / GBFFT_INVERSE (gbfft.h), Mode.hs:15-26
modeCode :: Mode -> CInt
modeCode Forward = -1
modeCode Reverse = 1
modeCode Inverse = 2

-- GBFFT_C32 / GBFFT_C64, Type.hs:28-30
dtypeCode :: NumericR e -> CInt
dtypeCode NumericRfloat32 = 0
dtypeCode NumericRfloat64 = 1

{-# INLINEABLE fft' #-}
fft' :: forall sh e.
        CInt
     -> Mode
     -> ShapeR sh
     -> NumericR e
     -> Array sh (Vec2 e)
     -> Par PTX (Future (Array sh (Vec2 e)))
fft' kind mode shR eR =
  let
      go :: ArrayR (Array sh (Vec2 e)) -> Array sh (Vec2 e) -> Par PTX (Future (Array sh (Vec2 e)))
      go aR ain = do
        let sh   = shape ain
            dims = map fromIntegral (reverse (shapeToList shR sh)) :: [Int64]  -- outermost first
        --
        aout    <- allocateRemote aR sh
        stream  <- asks ptxStream
        future  <- new
        liftPar $
          withArray eR ain stream   $ \d_in  -> do
           withArray eR aout stream $ \d_out -> do
             liftIO $ gbfft kind mode eR dims stream d_in d_out
        --
        put future aout
        return future
  in
  case eR of
    NumericRfloat32 -> go (ArrayR shR (eltR @(Complex Float)))
    NumericRfloat64 -> go (ArrayR shR (eltR @(Complex Double)))

-- Enqueue the transform on the Accelerate stream; a non-zero status becomes
-- an exception, as the cufft binding's errors did.
{-# INLINE gbfft #-}
gbfft :: CInt -> Mode -> NumericR e -> [Int64] -> Stream -> DevicePtr e -> DevicePtr e -> IO ()
gbfft kind mode eR dims stream d_in d_out =
  withLifetime stream $ \s ->
  withArrayLen dims   $ \rank pdims ->
  alloca              $ \pplan -> do
    r0 <- c_gbfft_plan_get pplan (fromIntegral rank) pdims kind (dtypeCode eR) precisionPlain
    when (r0 /= 0) $ throwIO (GbfftException (fromIntegral r0))
    plan <- peek pplan
    r <- c_gbfft_exec plan (modeCode mode) (castPtr (useDevicePtr d_in)) (castPtr (useDevicePtr d_out))
                      (castPtr (CUDA.useStream s))
    when (r /= 0) $ throwIO (GbfftException (fromIntegral r))

-- GBFFT_PLAIN: FP32 for Complex Float, FP64 for Complex Double
precisionPlain :: CInt
precisionPlain = 0
